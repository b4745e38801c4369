// CPU oracle: node-node hybrid coupling of hybridgrains2dnew, restated in plain
// C++ (FP64, serial branches of the reference).
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h).
#include "oracle_state.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

namespace hgo {

struct HybridState {
  MpmState *mpm = nullptr;
  DemState *dem = nullptr;
  std::vector<int> packed_dem, packed_mpm;
  std::vector<double> dem_mass_grid, dem_mom_grid, v_after, at_after,
      dem_pos_before;
  // ResamplingTools homogenisation accumulators (ResamplingTools.h)
  std::vector<double> homog_stress, homog_velocity, homog_mom, homog_mass;
};

inline bool nodeValid(const MpmState &s, unsigned ix, unsigned iy) {
  return ix <= s.nx && iy <= s.ny;
}

// Coupling.cpp:529-531
void copyPrePositionsFull(HybridState &h) { h.dem_pos_before = h.dem->q; }

// Coupling.cpp:22-140 (serial branch), allowCouplingPartiallyFilledCell and
// use_pre_position as passed by HybridGrains2DSim.cpp:141.
void rasterizeGrainMass(HybridState &h, bool allow_partial, bool use_pre) {
  MpmState &g = *h.mpm;
  DemState &d = *h.dem;
  const double hl = g.hl[0];
  const unsigned nn = g.nnodes();
  std::vector<int> coupled(d.n, 0);
  h.dem_mass_grid.assign(nn, 0.0);
  std::fill(g.hybridized.begin(), g.hybridized.end(), 0);
  for (int b = 0; b < d.n; ++b) {
    if (d.fixed[b]) continue;
    const std::vector<double> &qs = use_pre ? h.dem_pos_before : d.q;
    const V2 x{qs[3 * b], qs[3 * b + 1]};
    const Stencil st = stencilOf(g.basis, x, hl, g.gmin, g.h);
    bool all_pos = true;
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        if (!nodeValid(g, ix, iy)) continue;
        if (g.mass[g.flat(ix, iy)] <= 1.0e-6) all_pos = false;
      }
    if (!(all_pos || allow_partial)) continue;
    coupled[b] = 1;
    const double pm = d.M[3 * b];
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        if (!nodeValid(g, ix, iy)) continue;
        const double w = weightOf(g.basis, x, hl, ix, iy, g.gmin, g.h);
        h.dem_mass_grid[g.flat(ix, iy)] += w * pm;
      }
  }
  h.packed_dem.clear();
  for (int b = 0; b < d.n; ++b)
    if (coupled[b] > 0) h.packed_dem.push_back(b);
  h.packed_mpm.clear();
  for (unsigned i = 0; i < nn; ++i)
    if (h.dem_mass_grid[i] > 0.0) h.packed_mpm.push_back((int)i);
}

// Coupling.cpp:287-363 (serial branch)
void rasterizeGrainMom(HybridState &h, bool use_pre) {
  MpmState &g = *h.mpm;
  DemState &d = *h.dem;
  const double hl = g.hl[0];
  h.dem_mom_grid.assign(2 * g.nnodes(), 0.0);
  for (int b : h.packed_dem) {
    if (d.fixed[b]) continue;
    const std::vector<double> &qs = use_pre ? h.dem_pos_before : d.q;
    const V2 x{qs[3 * b], qs[3 * b + 1]};
    const Stencil st = stencilOf(g.basis, x, hl, g.gmin, g.h);
    const V2 pm{d.M[3 * b] * d.v[3 * b], d.M[3 * b] * d.v[3 * b + 1]};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        if (!nodeValid(g, ix, iy)) continue;
        const double w = weightOf(g.basis, x, hl, ix, iy, g.gmin, g.h);
        const unsigned i = g.flat(ix, iy);
        h.dem_mom_grid[2 * i] += w * pm.x;
        h.dem_mom_grid[2 * i + 1] += w * pm.y;
      }
  }
}

// Coupling.cpp:533-579
void updateVelocitiesOnGrid(HybridState &h) {
  MpmState &g = *h.mpm;
  const unsigned nn = g.nnodes();
  h.v_after.assign(2 * nn, 0.0);
  h.at_after.assign(2 * nn, 0.0);
  for (int i : h.packed_mpm) {
    const double m_mpm = g.mass[i];
    const double m_dem = h.dem_mass_grid[i];
    const double msum = m_mpm + m_dem;
    const V2 lambda{
        (m_dem * g.mom_new[2 * i] - m_mpm * h.dem_mom_grid[2 * i]) / msum,
        (m_dem * g.mom_new[2 * i + 1] - m_mpm * h.dem_mom_grid[2 * i + 1]) /
            msum};
    g.mom_new[2 * i] -= lambda.x;
    g.mom_new[2 * i + 1] -= lambda.y;
    const V2 after{h.dem_mom_grid[2 * i] + lambda.x,
                   h.dem_mom_grid[2 * i + 1] + lambda.y};
    h.v_after[2 * i] = after.x / m_dem;
    h.v_after[2 * i + 1] = after.y / m_dem;
    h.at_after[2 * i] = lambda.x / m_dem;
    h.at_after[2 * i + 1] = lambda.y / m_dem;
  }
}

// HybridGrains2DSim.cpp:183-197
void updateHomogFactor(HybridState &h) {
  MpmState &g = *h.mpm;
  const unsigned nn = g.nnodes();
  for (unsigned i = 0; i < nn; ++i) g.homog[i] = g.mass[i] > 0.0 ? 1.0 : 0.0;
  for (int i : h.packed_mpm) g.homog[i] = 0.5;
}

// Coupling.cpp:468-527 (alpha_phase_1 = 1: FLIP)
void transferToGrain(HybridState &h, bool use_pre) {
  MpmState &g = *h.mpm;
  DemState &d = *h.dem;
  const double alpha = 1.0;
  const double hl = g.hl[0];
  for (int b : h.packed_dem) {
    if (d.fixed[b]) continue;
    const std::vector<double> &qs = use_pre ? h.dem_pos_before : d.q;
    const V2 x{qs[3 * b], qs[3 * b + 1]};
    const Stencil st = stencilOf(g.basis, x, hl, g.gmin, g.h);
    V2 vpic{0, 0}, at{0, 0};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        if (!nodeValid(g, ix, iy)) continue;
        const double w = weightOf(g.basis, x, hl, ix, iy, g.gmin, g.h);
        const unsigned i = g.flat(ix, iy);
        vpic = add(vpic, scl(w, V2{h.v_after[2 * i], h.v_after[2 * i + 1]}));
        at = add(at, scl(w, V2{h.at_after[2 * i], h.at_after[2 * i + 1]}));
      }
    const V2 vflip{d.v[3 * b] + at.x, d.v[3 * b + 1] + at.y};
    d.v[3 * b] = vpic.x * (1.0 - alpha) + vflip.x * alpha;
    d.v[3 * b + 1] = vpic.y * (1.0 - alpha) + vflip.y * alpha;
  }
}

// Coupling.cpp:581-591
void updatePositionsNodeNode(HybridState &h, double dt) {
  DemState &d = *h.dem;
  for (int b : h.packed_dem) {
    d.q[3 * b] = h.dem_pos_before[3 * b] + dt * d.v[3 * b];
    d.q[3 * b + 1] = h.dem_pos_before[3 * b + 1] + dt * d.v[3 * b + 1];
  }
}

// ResamplingTools.cpp:736-742, 815-821
void clearHomogenized(HybridState &h) {
  const unsigned nn = h.mpm->nnodes();
  h.homog_stress.assign(4 * nn, 0.0);
  h.homog_velocity.assign(2 * nn, 0.0);
}

// ResamplingTools.cpp:744-813: contact stress -(f r^T + r f^T)/2 of every
// circle-circle contact spread with uGIMP-style half-width h/4 using the
// continuum basis, divided by the cell area.
void homogenizeStress(HybridState &h) {
  MpmState &g = *h.mpm;
  DemState &d = *h.dem;
  const double cw = g.h;
  const double area = cw * cw;
  const double hl = cw * 0.25;
  for (int b = 0; b < d.n; ++b)
    for (auto &e : d.cache.cc.entries[b]) {
      const int b1 = e.first;
      const V2 p = e.second.contact_point;
      const V2 r{d.q[3 * b] - d.q[3 * b1], d.q[3 * b + 1] - d.q[3 * b1 + 1]};
      const V2 f = add(e.second.normal_force, e.second.friction_force);
      // -0.5 * (f r^T + r f^T), column-major
      const M2 frt{f.x * r.x, f.y * r.x, f.x * r.y, f.y * r.y};
      const M2 rft{r.x * f.x, r.y * f.x, r.x * f.y, r.y * f.y};
      const M2 sc = mscl(-0.5, madd(frt, rft));
      const Stencil st = stencilOf(g.basis, p, hl, g.gmin, g.h);
      for (unsigned iy = st.y0; iy <= st.y1; ++iy)
        for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
          const double w = weightOf(g.basis, p, hl, ix, iy, g.gmin, g.h);
          const unsigned i = g.flat(ix, iy);
          const M2 add_ = mdiv(mscl(w, sc), area);
          h.homog_stress[4 * i] += add_.a00;
          h.homog_stress[4 * i + 1] += add_.a10;
          h.homog_stress[4 * i + 2] += add_.a01;
          h.homog_stress[4 * i + 3] += add_.a11;
        }
    }
}

// ResamplingTools.cpp:830-884
void homogenizeVelocity(HybridState &h) {
  MpmState &g = *h.mpm;
  DemState &d = *h.dem;
  const unsigned nn = g.nnodes();
  h.homog_mom.assign(2 * nn, 0.0);
  h.homog_mass.assign(nn, 0.0);
  const double hl = g.h * 0.25;
  for (int b = 0; b < d.n; ++b) {
    if (d.fixed[b]) continue;
    const double mass = d.M[3 * b];
    const V2 vel{d.v[3 * b], d.v[3 * b + 1]};
    const V2 pos{d.q[3 * b], d.q[3 * b + 1]};
    const Stencil st = stencilOf(g.basis, pos, hl, g.gmin, g.h);
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(g.basis, pos, hl, ix, iy, g.gmin, g.h);
        const unsigned i = g.flat(ix, iy);
        // weight * mass * velocity
        h.homog_mom[2 * i] += w * mass * vel.x;
        h.homog_mom[2 * i + 1] += w * mass * vel.y;
        h.homog_mass[i] += w * mass;
      }
  }
  for (unsigned i = 0; i < nn; ++i)
    if (h.homog_mass[i] > 0.0) {
      h.homog_velocity[2 * i] += h.homog_mom[2 * i] / h.homog_mass[i];
      h.homog_velocity[2 * i + 1] += h.homog_mom[2 * i + 1] / h.homog_mass[i];
    }
}

// HybridGrains2DSim.cpp:116-220: one prediction-correction-advection
// node-node step (resampling and zone relabelling excluded).
void hybridStep(HybridState &h, double dt) {
  const bool use_pre = true;
  copyPrePositionsFull(h);
  mpmPhase0(*h.mpm);
  rasterizeGrainMass(h, false, use_pre);
  demFlow(*h.dem, dt, true); // DiscreteIntegrator.cpp:99-116
  mpmPhase1(*h.mpm, dt);
  rasterizeGrainMom(h, use_pre);
  updateVelocitiesOnGrid(h);
  updateHomogFactor(h);
  transferToGrain(h, use_pre);
  mpmPhase2(*h.mpm, dt);
  updatePositionsNodeNode(h, dt);
}

} // namespace hgo

using namespace hgo;

extern "C" {

void *hgo_hybrid_create(void *mpm, void *dem) {
  HybridState *h = new HybridState();
  h->mpm = static_cast<MpmState *>(mpm);
  h->dem = static_cast<DemState *>(dem);
  clearHomogenized(*h);
  return h;
}

void hgo_hybrid_destroy(void *h) { delete static_cast<HybridState *>(h); }

// flags bit0: accumulate homogenized stress, bit1: homogenized velocity, each
// step after the coupling step (HybridGrains2DSim.cpp:545-556).
void hgo_hybrid_step(void *hp, double dt, int nsteps, int flags) {
  HybridState &h = *static_cast<HybridState *>(hp);
  for (int k = 0; k < nsteps; ++k) {
    hybridStep(h, dt);
    if (flags & 1) homogenizeStress(h);
    if (flags & 2) homogenizeVelocity(h);
  }
}

void hgo_hybrid_clear_homogenized(void *hp) {
  clearHomogenized(*static_cast<HybridState *>(hp));
}

int hgo_hybrid_num_packed(void *hp, int which) {
  HybridState &h = *static_cast<HybridState *>(hp);
  return which == 0 ? (int)h.packed_dem.size() : (int)h.packed_mpm.size();
}

void hgo_hybrid_get(void *hp, int *packed_dem, int *packed_mpm,
                    double *dem_mass_grid, double *dem_mom_grid,
                    double *v_after, double *at_after, double *homog_factor,
                    double *homog_stress, double *homog_velocity) {
  HybridState &h = *static_cast<HybridState *>(hp);
  const size_t nn = h.mpm->nnodes();
  auto cp = [](auto *dst, const auto &src) {
    if (dst && !src.empty())
      std::memcpy(dst, src.data(), sizeof(src[0]) * src.size());
  };
  cp(packed_dem, h.packed_dem);
  cp(packed_mpm, h.packed_mpm);
  cp(dem_mass_grid, h.dem_mass_grid);
  cp(dem_mom_grid, h.dem_mom_grid);
  cp(v_after, h.v_after);
  cp(at_after, h.at_after);
  if (homog_factor) std::memcpy(homog_factor, h.mpm->homog.data(), sizeof(double) * nn);
  cp(homog_stress, h.homog_stress);
  cp(homog_velocity, h.homog_velocity);
}

} // extern "C"
