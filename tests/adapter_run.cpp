// Drives the C++ adapters of include/ccd_gb300_reference.hpp as a reference
// program would: the CTCD forwarders on single stencils, then the k-DOP and
// AABB broad-phase adapters and the CTCD narrow-phase adapter on meshes, all
// through libccd_gb300.so.  Test infrastructure (tests/test_adapters_run_gpu.py
// writes the input and checks the output against the golden fixtures).
//
// Input (text, numbers in C99 hex-float or decimal form):
//   kat <n>, then n lines: <kind: vf|ee|ve|vv> <eta> <3 x points numbers>
//   mesh <name> <nv> <nf> <eta> <n_fixed>, then lines of 3nv start and 3nv end
//   coordinates, 3nf face indices and n_fixed vertex indices
// Output, one record per line:
//   kat <i> <hit> <t as %a>
//   cand <name> <kdop|aabb|kdop_fixed|aabb_fixed> <vf|ee> <4 indices>   (set order)
//   count <name> <label> <n_vf> <n_ee>
//   hit <name> <vf|ee> <4 indices>   (colliding stencils of the k-DOP candidates)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "ccd_gb300_reference.hpp"

static double next_number(FILE *f) {
  char buf[64];
  if (fscanf(f, "%63s", buf) != 1) {
    fprintf(stderr, "unexpected end of input\n");
    exit(2);
  }
  return strtod(buf, nullptr);
}

static void run_kat(FILE *in) {
  int n = (int)next_number(in);
  for (int i = 0; i < n; i++) {
    char kind[8];
    if (fscanf(in, "%7s", kind) != 1) exit(2);
    const double eta = next_number(in);
    const int npts = (!strcmp(kind, "vf") || !strcmp(kind, "ee")) ? 8 : (!strcmp(kind, "ve") ? 6 : 4);
    std::vector<Eigen::Vector3d> p((size_t)npts);
    for (int k = 0; k < npts; k++) {
      const double x = next_number(in), y = next_number(in), z = next_number(in);
      p[(size_t)k] = Eigen::Vector3d(x, y, z);
    }
    double t = -1.0;
    bool hit;
    if (!strcmp(kind, "vf"))
      hit = ccd_gb300::vertexFaceCTCD(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], eta, t);
    else if (!strcmp(kind, "ee"))
      hit = ccd_gb300::edgeEdgeCTCD(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], eta, t);
    else if (!strcmp(kind, "ve"))
      hit = ccd_gb300::vertexEdgeCTCD(p[0], p[1], p[2], p[3], p[4], p[5], eta, t);
    else
      hit = ccd_gb300::vertexVertexCTCD(p[0], p[1], p[2], p[3], eta, t);
    printf("kat %d %d %a\n", i, hit ? 1 : 0, t);
  }
}

static void run_mesh(FILE *in) {
  char name[64];
  if (fscanf(in, "%63s", name) != 1) exit(2);
  const int nv = (int)next_number(in), nf = (int)next_number(in);
  const double eta = next_number(in);
  const int nfixed = (int)next_number(in);
  Eigen::VectorXd qs(3 * nv), qe(3 * nv);
  for (int i = 0; i < 3 * nv; i++) qs[i] = next_number(in);
  for (int i = 0; i < 3 * nv; i++) qe[i] = next_number(in);
  Mesh m;
  m.vertices = qe;
  m.faces.resize(3, nf);
  for (int f = 0; f < nf; f++)
    for (int j = 0; j < 3; j++) m.faces(j, f) = (int)next_number(in);
  std::set<int> fixed, none;
  for (int i = 0; i < nfixed; i++) fixed.insert((int)next_number(in));
  History h(qs);
  h.finishHistory(qe);

  ccd_gb300::GpuKDOPBroadPhase kdop;
  ccd_gb300::GpuAABBBroadPhase aabb;
  std::set<VertexFaceStencil> kvf;
  std::set<EdgeEdgeStencil> kee;
  const struct {
    BroadPhase *bp;
    const char *label;
    const std::set<int> *fx;
  } runs[4] = {{&kdop, "kdop", &none}, {&aabb, "aabb", &none}, {&kdop, "kdop_fixed", &fixed},
               {&aabb, "aabb_fixed", &fixed}};
  for (const auto &r : runs) {
    std::set<VertexFaceStencil> vfs;
    std::set<EdgeEdgeStencil> ees;
    r.bp->findCollisionCandidates(h, m, eta, vfs, ees, *r.fx);
    printf("count %s %s %zu %zu\n", name, r.label, vfs.size(), ees.size());
    for (const auto &s : vfs) printf("cand %s %s vf %d %d %d %d\n", name, r.label, s.p, s.q0, s.q1, s.q2);
    for (const auto &s : ees) printf("cand %s %s ee %d %d %d %d\n", name, r.label, s.p0, s.p1, s.q0, s.q1);
    if (!strcmp(r.label, "kdop")) {
      kvf = vfs;
      kee = ees;
    }
  }
  // The narrow phase on the k-DOP candidates, each with the scene's eta.
  std::set<std::pair<VertexFaceStencil, double> > cvf;
  std::set<std::pair<EdgeEdgeStencil, double> > cee;
  for (const auto &s : kvf) cvf.insert(std::make_pair(s, eta));
  for (const auto &s : kee) cee.insert(std::make_pair(s, eta));
  ccd_gb300::GpuCTCDNarrowPhase narrow;
  std::set<VertexFaceStencil> hvf;
  std::set<EdgeEdgeStencil> hee;
  narrow.findCollisions(h, cvf, cee, hvf, hee);
  for (const auto &s : hvf) printf("hit %s vf %d %d %d %d\n", name, s.p, s.q0, s.q1, s.q2);
  for (const auto &s : hee) printf("hit %s ee %d %d %d %d\n", name, s.p0, s.p1, s.q0, s.q1);
}

int main(int argc, char **argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <input>\n", argv[0]);
    return 2;
  }
  FILE *in = fopen(argv[1], "r");
  if (!in) return 2;
  char word[16];
  try {
    while (fscanf(in, "%15s", word) == 1) {
      if (!strcmp(word, "kat"))
        run_kat(in);
      else if (!strcmp(word, "mesh"))
        run_mesh(in);
      else
        return 2;
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  fclose(in);
  return 0;
}
