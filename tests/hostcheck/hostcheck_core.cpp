// Host build of the device CTCD core (csrc/ccd_ctcd64.h) for the CPU tests:
// the same source the CUDA kernels compile, checked against the oracle here.
#include <cmath>
#include <cstdint>

#include "../../collisiondetection_gb300/csrc/ccd_ctcd64.h"

extern "C" void hc_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit,
                         double *t, uint8_t *status) {
  static const int width[4] = {24, 24, 18, 12};
  for (int64_t i = 0; i < n; i++) {
    const double *xi = x + i * width[kind];
    double e = eta_per_test ? eta[i] : eta[0];
    uint8_t st = 0;
    bool h;
    switch (kind) {
      case 0: h = ccd::vf_ctcd(xi, e, t[i], st); break;
      case 1: h = ccd::ee_ctcd(xi, e, t[i], st); break;
      case 2: h = ccd::ve_ctcd(xi, e, t[i], st); break;
      default: h = ccd::vv_ctcd(xi, e, t[i]); break;
    }
    hit[i] = h;
    status[i] = st;
  }
}

#include "../../collisiondetection_gb300/csrc/ccd_cull32.h"

// 1 where the FP32 stage rejects the row (kinds 0, 1 and 2).
extern "C" void hc_cull(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *rej) {
  const int w = kind == 2 ? 18 : 24;
  for (int64_t i = 0; i < n; i++) {
    const double *xi = x + i * w;
    double e = eta_per_test ? eta[i] : eta[0];
    rej[i] = kind == 0 ? ccd::vf_rejects(xi, e) : (kind == 1 ? ccd::ee_rejects(xi, e) : ccd::ve_rejects(xi, e));
  }
}
