// CPU oracle: penalty-DEM disk step of rigidbody2d, restated in plain C++
// (FP64, serial, like the reference).
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). The collision cache, the
// broadphase (std::map voxels + std::set of candidate pairs) and the force
// loop keep the reference's data structures and iteration orders, so that the
// floating-point summation order of body forces is the reference's.
#include "oracle_state.h"

#include <algorithm>
#include <cstring>
#include <limits>
#include <map>
#include <set>
#include <utility>
#include <vector>

namespace hgo {

struct AABB {
  V2 mn, mx;
};

// SpatialGrid.cpp:14-19
inline bool overlaps(const AABB &a, const AABB &b) {
  return (a.mx.x >= b.mn.x && a.mx.y >= b.mn.y) &&
         (b.mx.x >= a.mn.x && b.mx.y >= a.mn.y);
}

// SpatialGrid.cpp:54-88
void initializeSpatialGrid(const std::vector<AABB> &aabbs, double h_scale,
                           V2 &min_coord, unsigned dims[2], double &h) {
  const double inf = std::numeric_limits<double>::infinity();
  min_coord = {inf, inf};
  V2 max_coord{-inf, -inf};
  for (const AABB &a : aabbs) {
    min_coord = {std::min(min_coord.x, a.mn.x), std::min(min_coord.y, a.mn.y)};
    max_coord = {std::max(max_coord.x, a.mx.x), std::max(max_coord.y, a.mx.y)};
  }
  min_coord = {min_coord.x - 2.0e-6, min_coord.y - 2.0e-6};
  max_coord = {max_coord.x + 2.0e-6, max_coord.y + 2.0e-6};
  V2 delta{0.0, 0.0};
  for (const AABB &a : aabbs)
    delta = {delta.x + (a.mx.x - a.mn.x), delta.y + (a.mx.y - a.mn.y)};
  h = std::max(delta.x, delta.y) / (double)aabbs.size();
  h *= h_scale;
  dims[0] = (unsigned)std::ceil((max_coord.x - min_coord.x) / h);
  dims[1] = (unsigned)std::ceil((max_coord.y - min_coord.y) / h);
}

// SpatialGrid.cpp:30-52, 90-118
void getPotentialOverlaps(const std::vector<AABB> &aabbs, double h_scale,
                          std::set<std::pair<unsigned, unsigned>> &out,
                          double *h_out, unsigned *dims_out, V2 *origin_out) {
  V2 min_coord;
  unsigned dims[2];
  double h;
  initializeSpatialGrid(aabbs, h_scale, min_coord, dims, h);
  if (h_out) *h_out = h;
  if (dims_out) {
    dims_out[0] = dims[0];
    dims_out[1] = dims[1];
  }
  if (origin_out) *origin_out = min_coord;
  std::map<unsigned, std::vector<unsigned>> voxels;
  for (size_t i = 0; i < aabbs.size(); ++i) {
    const unsigned lx = (unsigned)(((aabbs[i].mn.x - min_coord.x) - 1.0e-6) / h);
    const unsigned ly = (unsigned)(((aabbs[i].mn.y - min_coord.y) - 1.0e-6) / h);
    const unsigned ux = (unsigned)(((aabbs[i].mx.x - min_coord.x) + 1.0e-6) / h);
    const unsigned uy = (unsigned)(((aabbs[i].mx.y - min_coord.y) + 1.0e-6) / h);
    for (unsigned x = lx; x <= ux; ++x)
      for (unsigned y = ly; y <= uy; ++y)
        voxels[x + dims[0] * y].emplace_back((unsigned)i);
  }
  for (const auto &vx : voxels) {
    const std::vector<unsigned> &ids = vx.second;
    for (size_t a = 0; a + 1 < ids.size(); ++a)
      for (size_t b = a + 1; b < ids.size(); ++b)
        if (overlaps(aabbs[ids[a]], aabbs[ids[b]]))
          out.insert(std::make_pair(ids[a], ids[b]));
  }
}

enum Kind { K_PLANE = 0, K_CC = 1, K_KIN = 2, K_DRUM = 3 };

struct Constraint {
  int kind;
  int i0, i1; // plane: body, plane index; kin: simulated body, fixed body
  V2 n, p;    // cc: normal and contact point from narrow phase
  double ra, rb;
};

inline V2 qpos(const DemState &s, int b) { return {s.q[3 * b], s.q[3 * b + 1]}; }
inline V2 vlin(const DemState &s, int b) { return {s.v[3 * b], s.v[3 * b + 1]}; }

// RigidBody2DSim::computeActiveSet (RigidBody2DSim.cpp:886-912) with q0 == q1
// as called from PenaltyImpactFrictionMap.cpp:43/311.
void computeActiveSet(const DemState &s, std::vector<Constraint> &out) {
  out.clear();
  // computeBodyBodyActiveSetSpatialGrid (RigidBody2DSim.cpp:1140-1178)
  std::vector<AABB> aabbs(s.n);
  for (int b = 0; b < s.n; ++b) { // CircleGeometry.cpp:22-30
    const V2 x = qpos(s, b);
    aabbs[b] = {{x.x - s.r[b], x.y - s.r[b]}, {x.x + s.r[b], x.y + s.r[b]}};
  }
  std::set<std::pair<unsigned, unsigned>> cand;
  if (s.n > 0) getPotentialOverlaps(aabbs, s.cell_scale, cand, nullptr, nullptr, nullptr);
  for (const auto &pr : cand) {
    // dispatchNarrowPhaseCollision (RigidBody2DSim.cpp:270-336)
    int a = (int)pr.first, b = (int)pr.second;
    if (s.fixed[a] && s.fixed[b]) continue;
    if (s.fixed[a]) std::swap(a, b);
    const V2 qa = qpos(s, a), qb = qpos(s, b);
    const double ra = s.r[a], rb = s.r[b];
    // CollisionDetectionUtilities.cpp:3-101 with q1 == q0: the quadratic and
    // linear coefficients vanish and the test reduces to c0 <= 0.
    const V2 d = sub(qa, qb);
    const double c0 = dot(d, d) - (ra + rb) * (ra + rb);
    if (!(c0 <= 0.0)) continue;
    const V2 nrm = normalized(sub(qa, qb));
    Constraint c;
    c.i0 = a;
    c.i1 = b;
    c.n = nrm;
    c.ra = ra;
    c.rb = rb;
    if (!s.fixed[b]) {
      c.kind = K_CC;
      c.p = add(qa, scl(ra / (ra + rb), sub(qb, qa)));
    } else {
      c.kind = K_KIN;
      c.p = {0, 0};
    }
    out.push_back(c);
  }
  // computeBodyPlaneActiveSetAllPairs (RigidBody2DSim.cpp:777-842)
  for (int pi = 0; pi < (int)s.planes.size(); ++pi) {
    const DemPlane &pl = s.planes[pi];
    for (int b = 0; b < s.n; ++b) {
      if (s.fixed[b]) continue;
      // StaticPlaneCircleConstraint.cpp:12-17
      if (dot(pl.n, sub(qpos(s, b), pl.x)) <= s.r[b]) {
        Constraint c;
        c.kind = K_PLANE;
        c.i0 = b;
        c.i1 = pi;
        c.n = pl.n;
        c.p = {0, 0};
        c.ra = s.r[b];
        c.rb = 0;
        out.push_back(c);
      }
    }
  }
  // computeBodyDrumActiveSetAllPairs (RigidBody2DSim.cpp:844-884)
  for (int di = 0; di < (int)s.drums.size(); ++di) {
    const DemDrum &dr = s.drums[di];
    for (int b = 0; b < s.n; ++b) {
      if (s.fixed[b]) continue;
      // StaticDrumCircleConstraint::isActive (StaticDrumCircleConstraint.cpp:7-13)
      const V2 d = sub(dr.x, qpos(s, b));
      const double gap = dr.r - s.r[b];
      if (sqnorm(d) >= gap * gap) {
        Constraint c;
        c.kind = K_DRUM;
        c.i0 = b;
        c.i1 = di;
        c.n = {0, 0};
        c.p = {0, 0};
        c.ra = s.r[b];
        c.rb = 0;
        out.push_back(c);
      }
    }
  }
}

inline V2 carryDeltaS(const Record *old, V2 vrel, V2 n, double dt) {
  V2 ds = old ? old->delta_s : V2{0, 0};
  ds = old ? add(ds, scl(dt, vrel)) : scl(dt, vrel);
  ds = sub(ds, scl(dot(n, ds), n));
  return ds;
}

// PenaltyImpactFrictionMap::updateCollisionCache
// (PenaltyImpactFrictionMap.cpp:28-294 unweighted, 296-599 weighted).
void updateCollisionCache(DemState &s, double dt, bool weighted) {
  s.old_cache.reset(s.n);
  std::vector<Constraint> as;
  computeActiveSet(s, as);
  for (const Constraint &c : as) {
    Record rec{};
    if (c.kind == K_PLANE) {
      const DemPlane &pl = s.planes[c.i1];
      const V2 x = qpos(s, c.i0);
      // StaticPlaneCircleConstraint.cpp:144-185
      rec.contact_point = sub(x, scl(c.ra, pl.n));
      rec.weight = weighted ? s.w[c.i0] : 1.0;
      rec.depth = std::min(0.0, dot(pl.n, sub(x, pl.x)) - c.ra);
      rec.n = pl.n;
      rec.r0 = scl(-c.ra, pl.n);
      const V2 t0{-rec.r0.y, rec.r0.x};
      // the static plane's collision point velocity is v + omega*t = 0
      const V2 arm = sub(rec.contact_point, pl.x);
      const V2 tp{-arm.y, arm.x};
      const V2 vplane{0.0 + 0.0 * tp.x, 0.0 + 0.0 * tp.y};
      rec.vrel = sub(add(vlin(s, c.i0), scl(s.v[3 * c.i0 + 2], t0)), vplane);
      const Record *old = s.cache.plane.find(c.i0, c.i1);
      rec.delta_s = carryDeltaS(old, rec.vrel, rec.n, dt);
      s.old_cache.plane.insert(c.i0, c.i1, rec);
    } else if (c.kind == K_DRUM) {
      const DemDrum &dr = s.drums[c.i1];
      const V2 x = qpos(s, c.i0);
      // StaticDrumCircleConstraint.cpp:100-159: the normal points from the
      // disk's centre to the drum's, the contact point is the disk's point
      // farthest from the drum's centre
      const V2 n = normalized(sub(dr.x, x));
      rec.contact_point = sub(x, scl(c.ra, n));
      rec.weight = weighted ? s.w[c.i0] : 1.0;
      rec.depth = std::min(0.0, -(norm(sub(dr.x, x)) - (dr.r - c.ra)));
      rec.n = n;
      rec.r0 = scl(-c.ra, n);
      const V2 t0{-rec.r0.y, rec.r0.x};
      // the static drum's collision point velocity is v + omega*t = 0
      const V2 arm = sub(rec.contact_point, dr.x);
      const V2 tp{-arm.y, arm.x};
      const V2 vdrum{0.0 + 0.0 * tp.x, 0.0 + 0.0 * tp.y};
      rec.vrel = sub(add(vlin(s, c.i0), scl(s.v[3 * c.i0 + 2], t0)), vdrum);
      const Record *old = s.cache.drum.find(c.i0, c.i1);
      rec.delta_s = carryDeltaS(old, rec.vrel, rec.n, dt);
      s.old_cache.drum.insert(c.i0, c.i1, rec);
    } else if (c.kind == K_CC) {
      const V2 qa = qpos(s, c.i0), qb = qpos(s, c.i1);
      rec.contact_point = c.p;
      rec.weight = weighted ? (s.w[c.i0] + s.w[c.i1]) * 0.5 : 1.0;
      // CircleCircleConstraint.cpp:171-233
      rec.depth = std::min(0.0, norm(sub(qa, qb)) - c.ra - c.rb);
      rec.n = c.n;
      rec.r0 = sub(c.p, qa);
      rec.r1 = sub(c.p, qb);
      const V2 t0{-rec.r0.y, rec.r0.x}, t1{-rec.r1.y, rec.r1.x};
      const V2 va = vlin(s, c.i0), vb = vlin(s, c.i1);
      rec.vrel = sub(sub(add(va, scl(s.v[3 * c.i0 + 2], t0)), vb),
                     scl(s.v[3 * c.i1 + 2], t1));
      const Record *old = s.cache.cc.find(c.i0, c.i1);
      rec.delta_s = carryDeltaS(old, rec.vrel, rec.n, dt);
      s.old_cache.cc.insert(c.i0, c.i1, rec);
    } else {
      const V2 qa = qpos(s, c.i0), qk = qpos(s, c.i1);
      // KinematicObjectCircleConstraint.cpp
      rec.contact_point = sub(qa, scl(c.ra, c.n));
      rec.weight = weighted ? s.w[c.i0] : 1.0;
      rec.depth = std::min(0.0, norm(sub(qa, qk)) - c.ra - c.rb);
      rec.n = c.n;
      rec.r0 = scl(-c.ra, c.n);
      const V2 t{-rec.r0.y, rec.r0.x};
      const V2 arm = sub(rec.contact_point, qk);
      const V2 tk{-arm.y, arm.x};
      const V2 vk = add(vlin(s, c.i1), scl(s.v[3 * c.i1 + 2], tk));
      rec.vrel = sub(add(vlin(s, c.i0), scl(s.v[3 * c.i0 + 2], t)), vk);
      const Record *old = s.cache.kin.find(c.i0, c.i1);
      rec.delta_s = carryDeltaS(old, rec.vrel, rec.n, dt);
      s.old_cache.kin.insert(c.i0, c.i1, rec);
    }
  }
  std::swap(s.cache, s.old_cache);
}

// PenaltyImpactFrictionMap.cpp:601-614
inline double secondRootOfQuadratic(double a, double b, double c, double ds) {
  if (b > 0.0) return (2.0 * c) / (-b - ds);
  return (-b + ds) / (2.0 * a);
}

// One contact of updateAnchorsAndAccumulateCollisionForces
// (PenaltyImpactFrictionMap.cpp:616-1081); returns the total force.
V2 contactForce(const DemState &s, Record &rec) {
  const double w = rec.weight;
  const V2 n = rec.n;
  const V2 deltas = rec.delta_s;
  const V2 vel = rec.vrel;
  const V2 vt = sub(vel, scl(dot(n, vel), n));
  const V2 vn = sub(vel, vt);
  const V2 normal_force =
      sub(scl(-s.kn * w * rec.depth, n), scl(0.5 * s.gn * w, vn));
  V2 friction_force = sub(scl(-s.kt * w, deltas), scl(0.5 * s.gt * w, vt));
  const double mu_fn = s.mu * norm(normal_force);
  const double ft = norm(friction_force);
  if (0.5 * s.gt * w * norm(vt) > mu_fn) {
    rec.delta_s = {0.0, 0.0};
    friction_force = scl(-0.5 * s.gt * w, vt);
    friction_force = normalized(friction_force);
    friction_force = scl(mu_fn, friction_force);
  } else if (ft > mu_fn) {
    const double a = s.kt * w * s.kt * w * sqnorm(deltas);
    const double b = s.kt * w * s.gt * w * dot(deltas, vt);
    const double c =
        0.25 * s.gt * w * s.gt * w * dot(vt, vt) - s.mu * s.mu * sqnorm(normal_force);
    const double dscr = b * b - 4 * a * c;
    const double dscr_sqrt = std::sqrt(dscr);
    const double root1 = secondRootOfQuadratic(a, b, c, dscr_sqrt);
    const V2 new_ds = scl(root1, deltas);
    friction_force = sub(scl(-s.kt * w, new_ds), scl(0.5 * s.gt * w, vt));
    rec.delta_s = new_ds;
  }
  rec.normal_force = normal_force;
  rec.friction_force = friction_force;
  return add(normal_force, friction_force);
}

void accumulateForces(DemState &s, std::vector<double> &F) {
  for (int b = 0; b < s.n; ++b) // circle vs plane
    for (auto &e : s.cache.plane.entries[b]) {
      const V2 f = contactForce(s, e.second);
      F[3 * b] += f.x;
      F[3 * b + 1] += f.y;
      F[3 * b + 2] += cross(e.second.r0, f);
    }
  for (int b = 0; b < s.n; ++b) // circle vs drum
    for (auto &e : s.cache.drum.entries[b]) {
      const V2 f = contactForce(s, e.second);
      F[3 * b] += f.x;
      F[3 * b + 1] += f.y;
      F[3 * b + 2] += cross(e.second.r0, f);
    }
  for (int b = 0; b < s.n; ++b) // circle vs circle
    for (auto &e : s.cache.cc.entries[b]) {
      const V2 f = contactForce(s, e.second);
      const int o = e.first;
      F[3 * b] += f.x;
      F[3 * b + 1] += f.y;
      F[3 * b + 2] += cross(e.second.r0, f);
      F[3 * o] -= f.x;
      F[3 * o + 1] -= f.y;
      F[3 * o + 2] -= cross(e.second.r1, f);
    }
  for (int b = 0; b < s.n; ++b) // kinematic circle vs circle
    for (auto &e : s.cache.kin.entries[b]) {
      const V2 f = contactForce(s, e.second);
      F[3 * b] += f.x;
      F[3 * b + 1] += f.y;
      F[3 * b + 2] += cross(e.second.r0, f);
    }
}

// PenaltyImpactFrictionMap::flow / flowWithWeights
// (PenaltyImpactFrictionMap.cpp:1083-1149)
void demFlow(DemState &s, double dt, bool weighted) {
  updateCollisionCache(s, dt, weighted);
  std::vector<double> F(3 * s.n, 0.0);
  // RigidBody2DSim::computeForce + NearEarthGravityForce.cpp:34-51
  for (int b = 0; b < s.n; ++b) {
    F[3 * b] += s.M[3 * b] * s.g.x;
    F[3 * b + 1] += s.M[3 * b] * s.g.y;
  }
  accumulateForces(s, F);
  for (int b = 0; b < s.n; ++b)
    if (s.fixed[b]) F[3 * b] = F[3 * b + 1] = F[3 * b + 2] = 0.0;
  for (int i = 0; i < 3 * s.n; ++i) s.v[i] = s.v[i] + (dt * s.Minv[i]) * F[i];
  for (int i = 0; i < 3 * s.n; ++i) s.q[i] = s.q[i] + dt * s.v[i];
}

// RigidBody2DState::updateCurrentMassUsingMassWeights
// (RigidBody2DState.cpp:1182-1200)
void demUpdateMasses(DemState &s) {
  s.M.resize(3 * s.n);
  s.Minv.resize(3 * s.n);
  for (int b = 0; b < s.n; ++b) {
    s.M[3 * b] = s.m0[b] * s.w[b];
    s.M[3 * b + 1] = s.m0[b] * s.w[b];
    s.M[3 * b + 2] = s.I0[b] * s.w[b];
    for (int k = 0; k < 3; ++k) s.Minv[3 * b + k] = 1.0 / s.M[3 * b + k];
  }
}

constexpr int REC_WIDTH = 22;

void packRecord(const Record &r, int kind, int i0, int i1, double *o) {
  o[0] = kind;
  o[1] = i0;
  o[2] = i1;
  o[3] = r.depth;
  o[4] = r.n.x;
  o[5] = r.n.y;
  o[6] = r.delta_s.x;
  o[7] = r.delta_s.y;
  o[8] = r.vrel.x;
  o[9] = r.vrel.y;
  o[10] = r.r0.x;
  o[11] = r.r0.y;
  o[12] = r.r1.x;
  o[13] = r.r1.y;
  o[14] = r.weight;
  o[15] = r.contact_point.x;
  o[16] = r.contact_point.y;
  o[17] = r.normal_force.x;
  o[18] = r.normal_force.y;
  o[19] = r.friction_force.x;
  o[20] = r.friction_force.y;
  o[21] = 0.0;
}

} // namespace hgo

using namespace hgo;

extern "C" {

// Bodies: q, v as 3N (x, y, theta); radii, masses (m = rho*pi*r^2) and
// inertias (I = m r^2 / 2, CircleGeometry.cpp:44-48) per body.
void *hgo_dem_create(int n, const double *q, const double *v, const double *r,
                     const double *m, const double *I,
                     const unsigned char *fixed, const double *g, double kn,
                     double kt, double gamman, double gammat, double mu,
                     double cell_scale) {
  DemState *s = new DemState();
  s->n = n;
  s->q.assign(q, q + 3 * n);
  s->v.assign(v, v + 3 * n);
  s->r.assign(r, r + n);
  s->m0.assign(m, m + n);
  s->I0.assign(I, I + n);
  s->w.assign(n, 1.0);
  s->fixed.assign(fixed, fixed + n);
  s->g = {g[0], g[1]};
  s->kn = kn;
  s->kt = kt;
  s->gn = gamman;
  s->gt = gammat;
  s->mu = mu;
  s->cell_scale = cell_scale;
  demUpdateMasses(*s);
  s->cache.reset(n);
  s->old_cache.reset(n);
  return s;
}

void hgo_dem_destroy(void *h) { delete static_cast<DemState *>(h); }

void hgo_dem_add_plane(void *h, const double *x, const double *n) {
  // RigidBody2DSceneParser.cpp:264: planes are built with n.normalized()
  static_cast<DemState *>(h)->planes.push_back(
      DemPlane{V2{x[0], x[1]}, normalized(V2{n[0], n[1]})});
}

void hgo_dem_add_drum(void *h, const double *x, double r) {
  static_cast<DemState *>(h)->drums.push_back(DemDrum{V2{x[0], x[1]}, r});
}

void hgo_dem_set_weights(void *h, const double *w) {
  DemState &s = *static_cast<DemState *>(h);
  s.w.assign(w, w + s.n);
  demUpdateMasses(s);
}

void hgo_dem_set_state(void *h, const double *q, const double *v) {
  DemState &s = *static_cast<DemState *>(h);
  if (q) s.q.assign(q, q + 3 * s.n);
  if (v) s.v.assign(v, v + 3 * s.n);
}

void hgo_dem_step(void *h, double dt, int nsteps, int weighted) {
  DemState &s = *static_cast<DemState *>(h);
  for (int k = 0; k < nsteps; ++k) demFlow(s, dt, weighted != 0);
}

void hgo_dem_get_state(void *h, double *q, double *v) {
  DemState &s = *static_cast<DemState *>(h);
  if (q) std::memcpy(q, s.q.data(), sizeof(double) * 3 * s.n);
  if (v) std::memcpy(v, s.v.data(), sizeof(double) * 3 * s.n);
}

int hgo_dem_record_width() { return REC_WIDTH; }

// All cached contacts: contacts with static objects (body-major; each
// body's plane contacts, then its drum contacts), circle-circle
// (body-major), kinematic (body-major), the order of the library's
// export. Returns the count; writes at most cap.
int hgo_dem_get_contacts(void *h, int cap, double *out) {
  DemState &s = *static_cast<DemState *>(h);
  int k = 0;
  auto emit_body = [&](TypeCache &tc, int kind, int b) {
    for (auto &e : tc.entries[b]) {
      if (k < cap) packRecord(e.second, kind, b, e.first, out + REC_WIDTH * k);
      ++k;
    }
  };
  auto emit = [&](TypeCache &tc, int kind) {
    for (int b = 0; b < s.n; ++b) emit_body(tc, kind, b);
  };
  for (int b = 0; b < s.n; ++b) {
    emit_body(s.cache.plane, K_PLANE, b);
    emit_body(s.cache.drum, K_DRUM, b);
  }
  emit(s.cache.cc, K_CC);
  emit(s.cache.kin, K_KIN);
  return k;
}

// SpatialGrid::getPotentialOverlaps on explicit AABBs. pairs gets (i, j)
// with i < j in std::set order; returns the count (writes at most cap).
int hgo_dem_candidate_pairs(int n, const double *aabb_min,
                            const double *aabb_max, double cell_scale, int cap,
                            int *pairs, double *h_out, unsigned *dims_out,
                            double *origin_out) {
  std::vector<AABB> aabbs(n);
  for (int i = 0; i < n; ++i)
    aabbs[i] = {{aabb_min[2 * i], aabb_min[2 * i + 1]},
                {aabb_max[2 * i], aabb_max[2 * i + 1]}};
  std::set<std::pair<unsigned, unsigned>> out;
  V2 origin{0, 0};
  if (n > 0) getPotentialOverlaps(aabbs, cell_scale, out, h_out, dims_out, &origin);
  if (origin_out) {
    origin_out[0] = origin.x;
    origin_out[1] = origin.y;
  }
  int k = 0;
  for (const auto &p : out) {
    if (k < cap) {
      pairs[2 * k] = (int)p.first;
      pairs[2 * k + 1] = (int)p.second;
    }
    ++k;
  }
  return k;
}

} // extern "C"
