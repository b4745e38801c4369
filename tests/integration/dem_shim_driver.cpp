// Drives the DEM shim of INTEGRATION.md (GpuPenaltyImpactFrictionMap) the
// way the reference's hybrid loop does (test infrastructure):
//
//   1. two steps through flowWithWeights;
//   2. the host changes some bodies' velocities and positions, as the
//      coupling does after every DEM step (Coupling.cpp:468-527, 581-591),
//      and two more steps;
//   3. bodies removed through RigidBody2DState::removeBodies (NaN marks and
//      deleteCacheEntries) and two added through addBody (enlargeCache), as
//      the resampling step does, and two more steps.
//
// Usage: dem_shim_driver <input> <output>. The input holds, little-endian:
// int64 n; double dt, kn, kt, gamman, gammat, mu, gx, gy; then q[3n], v[3n],
// r[n], m[n], I[n] as doubles and fixed[n] as bytes. The output holds, after
// each of the three stages, int64 n, q[3n], v[3n].
#include "reference_stubs.h"

#include "dem_shim.inc"

#include <cstdio>
#include <cstring>
#include <vector>

// The solver-side arguments of flowWithWeights are not used by the device
// map; complete types stand in for the reference's classes here.
class ScriptingCallback {};
class FlowableSystem {};
class ConstrainedSystem {};
class UnconstrainedMap {};
class FrictionSolver {};

namespace {

bool read_all(const char *path, std::vector<char> &buf) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  char tmp[1 << 16];
  size_t k;
  while ((k = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + k);
  std::fclose(f);
  return true;
}

void write_stage(FILE *f, const RigidBody2DState &s) {
  const int64_t n = s.nbodies();
  std::fwrite(&n, sizeof n, 1, f);
  std::fwrite(s.q().data(), sizeof(double), 3 * n, f);
  std::fwrite(s.v().data(), sizeof(double), 3 * n, f);
}

// RigidBody2DSim::flowWithWeight's use of the map (RigidBody2DSim.cpp:1041-1069):
// the state's q, v and mass weights in, the new q, v swapped in
void step(ImpactFrictionMap &map, RigidBody2DState &s, double dt) {
  ScriptingCallback cb;
  FlowableSystem fsys;
  ConstrainedSystem csys;
  UnconstrainedMap umap;
  FrictionSolver solver;
  VectorXs q1, v1;
  map.flowWithWeights(cb, fsys, csys, umap, solver, 0u, dt, 0.0, 0.0, false, s.q(), s.v(),
                      s.massWeights(), q1, v1);
  s.q() = q1;
  s.v() = v1;
}

} // namespace

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  std::vector<char> in;
  if (!read_all(argv[1], in)) return 3;
  const char *p = in.data();
  int64_t n;
  std::memcpy(&n, p, 8);
  p += 8;
  double prm[8];
  std::memcpy(prm, p, sizeof prm);
  p += sizeof prm;
  const double dt = prm[0];
  std::vector<double> q(3 * n), v(3 * n), r(n), m(n), I(n);
  std::vector<uint8_t> fixed(n);
  for (auto *a : {&q, &v}) {
    std::memcpy(a->data(), p, 8 * a->size());
    p += 8 * a->size();
  }
  for (auto *a : {&r, &m, &I}) {
    std::memcpy(a->data(), p, 8 * a->size());
    p += 8 * a->size();
  }
  std::memcpy(fixed.data(), p, n);

  hg_context *ctx = nullptr;
  if (hg_context_create(0, &ctx) != HG_OK) return 4;
  hg_dem_desc d{};
  d.kn = prm[1];
  d.kt = prm[2];
  d.gamman = prm[3];
  d.gammat = prm[4];
  d.mu = prm[5];
  d.gravity[0] = prm[6];
  d.gravity[1] = prm[7];
  d.cell_scale = 1.0;
  d.num_planes = 1;
  d.planes[0].n[1] = 1.0; // the floor y = 0
  d.capacity = n + 16;
  d.contact_capacity = 8 * (n + 16);

  RigidBody2DState state;
  for (int64_t i = 0; i < n; ++i)
    state.add_circle(&q[3 * i], &v[3 * i], r[i], m[i], I[i], fixed[i] != 0, nullptr);
  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 5;
  int rc = 0;
  try {
    GpuPenaltyImpactFrictionMap map(state, ctx, d);
    step(map, state, dt);
    step(map, state, dt);
    write_stage(out, state);
    for (unsigned i = 0; i < state.nbodies(); ++i) {
      if (i % 5 == 0) state.v()(3 * i + 1) = -0.1;
      if (i % 7 == 0) state.q()(3 * i) += 1.0e-5;
    }
    step(map, state, dt);
    step(map, state, dt);
    write_stage(out, state);
    std::vector<unsigned> gone;
    for (unsigned i = 0; i < state.nbodies(); ++i)
      if (i % 11 == 3) gone.push_back(i);
    state.remove_marked(gone, &map);
    const double qa[3] = {0.5, 0.5, 0.0}, qb[3] = {0.6, 0.5, 0.0}, va[3] = {0.0, 0.0, 0.0};
    state.add_circle(qa, va, 1.0e-3, m[0], I[0], false, &map);
    state.add_circle(qb, va, 1.0e-3, m[0], I[0], false, &map);
    step(map, state, dt);
    step(map, state, dt);
    write_stage(out, state);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    rc = 6;
  }
  std::fclose(out);
  hg_context_destroy(ctx);
  return rc;
}
