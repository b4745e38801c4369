// CPU oracle: state containers shared by the MPM, DEM and coupling oracles.
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h).
#pragma once

#include "oracle_common.h"

#include <utility>
#include <vector>

namespace hgo {

enum Basis { LINEAR = 0, UGIMP = 1 };

struct MpmPlane { // mpmgrains2d/StaticPlane.h:6-22
  V2 x, n;
  int sticking; // 0 SLIDING, 1 STICKING
  double lower_bound;
};

// SimulationState = PhysicsGrid + MaterialPoints + material scalars
// (mpmgrains2d/SimulationState.h, PhysicsGrid.h, MaterialPoints.h:111-152).
struct MpmState {
  V2 gmin, gmax;
  double h = 0.0;
  unsigned nx = 0, ny = 0; // cell_count
  std::vector<double> mass, mom, mom_new, force, vel, acc, coupling_force,
      homog;
  std::vector<int> hybridized;
  int np = 0;
  std::vector<double> q, v, m, vol, hl, be, J, sigma, velgrad;
  std::vector<int> jh;
  std::vector<unsigned char> kin;
  double mu = 0, kappa = 0, dp_alpha = 0, flip_alpha = 0;
  V2 g{0, 0};
  int basis = LINEAR;
  std::vector<MpmPlane> planes;
  int nthreads = 1;

  unsigned nnodes() const { return (nx + 1) * (ny + 1); }
  unsigned flat(unsigned ix, unsigned iy) const { return iy * (nx + 1) + ix; }
  V2 qp(int p) const { return {q[2 * p], q[2 * p + 1]}; }
  M2 bep(int p) const {
    return {be[4 * p], be[4 * p + 1], be[4 * p + 2], be[4 * p + 3]};
  }
  void setbe(int p, M2 a) {
    be[4 * p] = a.a00;
    be[4 * p + 1] = a.a10;
    be[4 * p + 2] = a.a01;
    be[4 * p + 3] = a.a11;
  }
  M2 sigp(int p) const {
    return {sigma[4 * p], sigma[4 * p + 1], sigma[4 * p + 2],
            sigma[4 * p + 3]};
  }
};

struct Stencil {
  unsigned x0, y0, x1, y1; // inclusive node range
};

Stencil stencilOf(int basis, V2 x, double hl, V2 gmin, double h);
double weightOf(int basis, V2 x, double hl, unsigned ix, unsigned iy, V2 gmin,
                double h);
V2 weightGradOf(int basis, V2 x, double hl, unsigned ix, unsigned iy, V2 gmin,
                double h);
void mpmPhase0(MpmState &s);
void mpmPhase1(MpmState &s, double dt);
void mpmPhase2(MpmState &s, double dt);

// ---- DEM --------------------------------------------------------------------

struct Record { // PenaltyImpactFrictionMap.h:10-158 (union of the fields)
  double depth;
  V2 n, delta_s, vrel, r0, r1;
  double weight;
  V2 contact_point, normal_force, friction_force;
};

struct DemPlane { // rigidbody2d/RigidBody2DStaticPlane.h (static: v = 0, omega = 0)
  V2 x, n;
};

struct DemDrum { // rigidbody2d/RigidBody2DStaticDrum.h:6-33 (static: v = 0, omega = 0)
  V2 x;
  double r;
};

// CollisionTypeCache (PenaltyImpactFrictionMap.h:167-273): one list per body.
struct TypeCache {
  std::vector<std::vector<std::pair<int, Record>>> entries;
  int count = 0;
  void reset(int n) {
    entries.assign(n, {});
    count = 0;
  }
  Record *find(int i0, int i1) {
    if (count == 0) return nullptr;
    for (auto &e : entries[i0])
      if (e.first == i1) return &e.second;
    return nullptr;
  }
  void insert(int i0, int i1, const Record &r) {
    entries[i0].emplace_back(i1, r);
    ++count;
  }
};

struct Cache { // CollisionCache (PenaltyImpactFrictionMap.h): the circle kinds
  TypeCache plane, drum, cc, kin;
  void reset(int n) {
    plane.reset(n);
    drum.reset(n);
    cc.reset(n);
    kin.reset(n);
  }
};

struct DemState {
  int n = 0;
  std::vector<double> q, v, r, m0, I0, w, M, Minv; // M, Minv: 3 per body
  std::vector<unsigned char> fixed;
  std::vector<DemPlane> planes;
  std::vector<DemDrum> drums;
  V2 g{0, 0};
  double kn = 0, kt = 0, gn = 0, gt = 0, mu = 0, cell_scale = 1.0;
  Cache cache, old_cache;
};

void demFlow(DemState &s, double dt, bool weighted);
void demUpdateMasses(DemState &s);

} // namespace hgo
