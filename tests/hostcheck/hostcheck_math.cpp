// Host build of the device math (csrc/ccd_math.h) for the CPU tests.
#include <cmath>
#include <cstdint>

#include "../../collisiondetection_gb300/csrc/ccd_math.h"

extern "C" {
void hc_log(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = ccd::cr_log(x[i]);
}
void hc_exp(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = ccd::cr_exp(x[i]);
}
void hc_libm_log(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = std::log(x[i]);
}
void hc_libm_exp(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = std::exp(x[i]);
}
}

extern "C" {
void hc_log_slow(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = ccd::cr_log_slow(x[i]);
}
void hc_exp_slow(const double *x, double *y, int64_t n) {
  for (int64_t i = 0; i < n; i++) y[i] = ccd::cr_exp_slow(x[i]);
}
}
