// Node-node hybrid coupling (hybridgrains2dnew/Coupling.cpp,
// HybridGrains2DSim.cpp:116-220) over the FP64 MPM path and the DEM path.
//
// Compiled with --fmad=false. Grain-to-grid scatters use FP64 atomics (sums
// differ from the serial reference in order only); the packed grain and node
// lists are built with a scan, so they keep the reference's stable-partition
// order (Coupling.cpp:113-127). With a MIXED (FP32) MPM bulk the grains' and
// contacts' stencil weights are FP32 (for_stencil_weights32) over the same
// FP64 stencils; the grids and the exchange stay FP64.
//
// Kernels:
//   kc_grain_mass     rasterizeGrainMass (Coupling.cpp:22-140)
//   kc_flag_nodes /   std::stable_partition of grains and nodes
//   kc_pack             (Coupling.cpp:113-127)
//   kc_grain_mom      rasterizeGrainMom (Coupling.cpp:287-363)
//   kc_update_nodes   updateVelocitiesOnGrid (Coupling.cpp:533-579) and the
//                     homog_factor loop (HybridGrains2DSim.cpp:183-197), over
//                     every node
//   kc_transfer       transferToGrain, FLIP with alpha = 1 (Coupling.cpp:468-527),
//                     then updatePositions_node_node (Coupling.cpp:581-591)
//   kc_hstress        ResamplingTools::homogenizeStress (ResamplingTools.cpp:744-813)
//   kc_hvel_scatter / ResamplingTools::homogenizeVelocity
//   kc_hvel_finish      (ResamplingTools.cpp:830-884)
#include "hg_internal.cuh"
#include "mpm_basis.cuh"

#include <algorithm>

namespace hg {

namespace {

struct GridGeom {
  int basis, nx, ny;
  double gx, gy, h;
  double inv_h;
};

GridGeom geom(const hg_mpm *m) {
  return GridGeom{m->p.basis, m->p.nx, m->p.ny, m->p.gmin[0], m->p.gmin[1], m->p.h, m->p.inv_h};
}

// The grid weights of a grain's or contact's stencil: FP32 (W32, for a MIXED
// bulk) or FP64 in the reference's operation order (an FP64 bulk).
template <bool W32, class F>
__device__ __forceinline__ void stencil_weights(const GridGeom &G, double x, double y, double hl,
                                                int x0, int y0, int x1, int y1, F &&f) {
  if (W32)
    for_stencil_weights32(G.basis, x, y, hl, x0, y0, x1, y1, G.gx, G.gy, G.h, G.inv_h, f);
  else
    for_stencil_weights(G.basis, x, y, hl, x0, y0, x1, y1, G.gx, G.gy, G.h, f);
}

__device__ __forceinline__ bool node_ok(const GridGeom &G, int ix, int iy) {
  return ix >= 0 && iy >= 0 && ix <= G.nx && iy <= G.ny;
}

// M: the MPM node mass type (double for an FP64 object, float for MIXED,
// where it is the P2G sum of this step before the grid update).
template <typename M>
__global__ void kc_grain_mass(GridGeom G, int64_t nb, const double *__restrict__ pos,
                              const double *__restrict__ hl0, const uint8_t *__restrict__ fixed,
                              const double *__restrict__ m0, const double *__restrict__ w,
                              const M *__restrict__ g_mass, double *dem_mass,
                              int32_t *coupled) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  coupled[b] = 0;
  if (fixed[b]) return;
  const double hl = hl0[0]; // points.hl(0): the first material point's extent
  const double x = pos[3 * b], y = pos[3 * b + 1];
  int x0, y0, x1, y1;
  stencil64(G.basis, x, y, hl, G.gx, G.gy, G.h, x0, y0, x1, y1);
  bool all_pos = true;
  for (int iy = y0; iy <= y1; ++iy)
    for (int ix = x0; ix <= x1; ++ix) {
      if (!node_ok(G, ix, iy)) continue;
      if ((double)g_mass[(int64_t)iy * (G.nx + 1) + ix] <= 1.0e-6) all_pos = false;
    }
  if (!all_pos) return;
  coupled[b] = 1;
  const double pm = m0[b] * w[b]; // RigidBody2DState::getTotalMass
  stencil_weights<sizeof(M) == sizeof(float)>(G, x, y, hl, x0, y0, x1, y1,
                      [&](int ix, int iy, double wt) {
                        if (!node_ok(G, ix, iy)) return;
                        atomicAdd(&dem_mass[(int64_t)iy * (G.nx + 1) + ix], wt * pm);
                      });
}

__global__ void kc_flag_nodes(int64_t nn, const double *__restrict__ dem_mass, int32_t *flag) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  flag[i] = dem_mass[i] > 0.0 ? 1 : 0;
}

// Stable partition: writes the indices with flag set, in index order.
__global__ void kc_pack(int64_t n, const int32_t *__restrict__ flag,
                        const int32_t *__restrict__ pos, int32_t *out, int32_t *count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    *count = pos[n];
    return;
  }
  if (flag[i]) out[pos[i]] = (int32_t)i;
}

template <bool W32>
__global__ void kc_grain_mom(GridGeom G, int64_t nb, const int32_t *__restrict__ coupled,
                             const double *__restrict__ pos,
                             const double *__restrict__ hl0, const uint8_t *__restrict__ fixed,
                             const double *__restrict__ m0, const double *__restrict__ w,
                             const double *__restrict__ v, double *dem_mom) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb;
       b += (int64_t)gridDim.x * blockDim.x) {
    if (!coupled[b] || fixed[b]) continue;
    const double hl = hl0[0];
    const double x = pos[3 * b], y = pos[3 * b + 1];
    int x0, y0, x1, y1;
    stencil64(G.basis, x, y, hl, G.gx, G.gy, G.h, x0, y0, x1, y1);
    const double pm = m0[b] * w[b];
    const double px = pm * v[3 * b], py = pm * v[3 * b + 1];
    stencil_weights<W32>(G, x, y, hl, x0, y0, x1, y1,
                        [&](int ix, int iy, double wt) {
                          if (!node_ok(G, ix, iy)) return;
                          const int64_t i = (int64_t)iy * (G.nx + 1) + ix;
                          atomicAdd(&dem_mom[2 * i], wt * px);
                          atomicAdd(&dem_mom[2 * i + 1], wt * py);
                        });
  }
}

// Every node: its homogenisation factor (HybridGrains2DSim.cpp:183-197: 1/2
// where the DEM has mass, else 1 where the MPM has), and on the coupled nodes
// (DEM mass > 0) updateVelocitiesOnGrid; v_after and a_after are zero
// elsewhere.
__global__ void kc_update_nodes(int64_t nn, const double *__restrict__ g_mass,
                                const double *__restrict__ dem_mass,
                                const double *__restrict__ dem_mom, double *g_mom_new,
                                double *v_after, double *a_after, double *homog) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double m_mpm = g_mass[i], m_dem = dem_mass[i];
    homog[i] = m_dem > 0.0 ? 0.5 : (m_mpm > 0.0 ? 1.0 : 0.0);
    if (!(m_dem > 0.0)) {
      v_after[2 * i] = v_after[2 * i + 1] = 0.0;
      a_after[2 * i] = a_after[2 * i + 1] = 0.0;
      continue;
    }
    const double msum = m_mpm + m_dem;
    const double lx = (m_dem * g_mom_new[2 * i] - m_mpm * dem_mom[2 * i]) / msum;
    const double ly = (m_dem * g_mom_new[2 * i + 1] - m_mpm * dem_mom[2 * i + 1]) / msum;
    g_mom_new[2 * i] -= lx;
    g_mom_new[2 * i + 1] -= ly;
    const double ax = dem_mom[2 * i] + lx, ay = dem_mom[2 * i + 1] + ly;
    v_after[2 * i] = ax / m_dem;
    v_after[2 * i + 1] = ay / m_dem;
    a_after[2 * i] = lx / m_dem;
    a_after[2 * i + 1] = ly / m_dem;
  }
}

// updateVelocitiesOnGrid (Coupling.cpp:533-579) on a MIXED grid: the MPM
// node momentum after the grid update is gm v (FP32 velocity and mass), the
// exchange lambda is formed in FP64 as in kc_update_nodes, and the node's
// velocity and acceleration (va: v, a) take p_new - lambda; the acceleration
// (p_new - p) / (m dt) loses lambda / (m dt). Nodes without MPM mass keep
// their zero velocity, as (p_new = 0) / m is never formed for them.
__global__ void kc_update_nodes_x(int64_t nn, const float *__restrict__ gm,
                                  const double *__restrict__ dem_mass,
                                  const double *__restrict__ dem_mom, double dt, float4 *va,
                                  double *v_after, double *a_after, double *homog) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double m_mpm = (double)gm[i], m_dem = dem_mass[i];
    homog[i] = m_dem > 0.0 ? 0.5 : (m_mpm > 0.0 ? 1.0 : 0.0); // as kc_update_nodes
    if (!(m_dem > 0.0)) {
      v_after[2 * i] = v_after[2 * i + 1] = 0.0;
      a_after[2 * i] = a_after[2 * i + 1] = 0.0;
      continue;
    }
    float4 g = va[i];
    const double px = m_mpm * (double)g.x, py = m_mpm * (double)g.y;
    const double msum = m_mpm + m_dem;
    const double lx = (m_dem * px - m_mpm * dem_mom[2 * i]) / msum;
    const double ly = (m_dem * py - m_mpm * dem_mom[2 * i + 1]) / msum;
    if (m_mpm > 0.0) {
      g.x = (float)((px - lx) / m_mpm);
      g.y = (float)((py - ly) / m_mpm);
      g.z = (float)((double)g.z - lx / (m_mpm * dt));
      g.w = (float)((double)g.w - ly / (m_mpm * dt));
      va[i] = g;
    }
    const double ax = dem_mom[2 * i] + lx, ay = dem_mom[2 * i + 1] + ly;
    v_after[2 * i] = ax / m_dem;
    v_after[2 * i + 1] = ay / m_dem;
    a_after[2 * i] = lx / m_dem;
    a_after[2 * i + 1] = ly / m_dem;
  }
}

__global__ void kc_set_scalar(double *dst, double v) { *dst = v; }

__global__ void kc_fill(double *dst, int64_t n, double v) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = v;
}

template <bool W32>
// transferToGrain (Coupling.cpp:468-527) and then, as nothing between them
// touches the grains, updatePositions_node_node (Coupling.cpp:581-591):
// q = q_before + dt v for every coupled grain (fixed ones keep their v)
__global__ void kc_transfer(GridGeom G, int64_t nb, const int32_t *__restrict__ coupled,
                            const double *__restrict__ pos,
                            const double *__restrict__ hl0, const uint8_t *__restrict__ fixed,
                            const double *__restrict__ v_after,
                            const double *__restrict__ a_after, double dt, double *v, double *q) {
  const double alpha = 1.0;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb;
       b += (int64_t)gridDim.x * blockDim.x) {
    if (!coupled[b]) continue;
    if (fixed[b]) {
      q[3 * b] = pos[3 * b] + dt * v[3 * b];
      q[3 * b + 1] = pos[3 * b + 1] + dt * v[3 * b + 1];
      continue;
    }
    const double hl = hl0[0];
    const double x = pos[3 * b], y = pos[3 * b + 1];
    int x0, y0, x1, y1;
    stencil64(G.basis, x, y, hl, G.gx, G.gy, G.h, x0, y0, x1, y1);
    double vpx = 0.0, vpy = 0.0, atx = 0.0, aty = 0.0;
    stencil_weights<W32>(G, x, y, hl, x0, y0, x1, y1,
                        [&](int ix, int iy, double wt) {
                          if (!node_ok(G, ix, iy)) return;
                          const int64_t i = (int64_t)iy * (G.nx + 1) + ix;
                          vpx = vpx + wt * v_after[2 * i];
                          vpy = vpy + wt * v_after[2 * i + 1];
                          atx = atx + wt * a_after[2 * i];
                          aty = aty + wt * a_after[2 * i + 1];
                        });
    const double fx = v[3 * b] + atx, fy = v[3 * b + 1] + aty;
    const double vx = vpx * (1.0 - alpha) + fx * alpha, vy = vpy * (1.0 - alpha) + fy * alpha;
    v[3 * b] = vx;
    v[3 * b + 1] = vy;
    q[3 * b] = pos[3 * b] + dt * vx;
    q[3 * b + 1] = pos[3 * b + 1] + dt * vy;
  }
}

template <bool W32>
__global__ void kc_hstress(GridGeom G, int64_t nb, const int32_t *__restrict__ off,
                           const double *__restrict__ rec, const double *__restrict__ q,
                           double *hs) {
  // circle-circle contacts occupy [off[nb], off[2 nb]) of the contact list
  const int s = off[nb], e = off[2 * nb];
  const double cw = G.h;
  const double area = cw * cw;
  const double hl = cw * 0.25;
  for (int64_t k = s + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < e;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double *r_ = rec + k * HG_DEM_RECORD_WIDTH;
    const int b0 = (int)r_[1], b1 = (int)r_[2];
    const double px = r_[15], py = r_[16];
    const double rx = q[3 * b0] - q[3 * b1], ry = q[3 * b0 + 1] - q[3 * b1 + 1];
    const double fx = r_[17] + r_[19], fy = r_[18] + r_[20];
    // -0.5 (f r^T + r f^T), column-major (00, 10, 01, 11)
    const double s00 = -0.5 * (fx * rx + rx * fx);
    const double s10 = -0.5 * (fy * rx + ry * fx);
    const double s01 = -0.5 * (fx * ry + rx * fy);
    const double s11 = -0.5 * (fy * ry + ry * fy);
    // FP64 bulk: the reference's (w s) / area per node. Mixed bulk: w (s /
    // area), one division per component and contact instead of one per node
    // (FP64 division is a long sequence on the FP64 pipe).
    const double d00 = W32 ? s00 / area : s00, d10 = W32 ? s10 / area : s10;
    const double d01 = W32 ? s01 / area : s01, d11 = W32 ? s11 / area : s11;
    int x0, y0, x1, y1;
    stencil64(G.basis, px, py, hl, G.gx, G.gy, G.h, x0, y0, x1, y1);
    stencil_weights<W32>(G, px, py, hl, x0, y0, x1, y1,
                        [&](int ix, int iy, double wt) {
                          if (!node_ok(G, ix, iy)) return;
                          const int64_t i = (int64_t)iy * (G.nx + 1) + ix;
                          atomicAdd(&hs[4 * i], W32 ? wt * d00 : wt * d00 / area);
                          atomicAdd(&hs[4 * i + 1], W32 ? wt * d10 : wt * d10 / area);
                          atomicAdd(&hs[4 * i + 2], W32 ? wt * d01 : wt * d01 / area);
                          atomicAdd(&hs[4 * i + 3], W32 ? wt * d11 : wt * d11 / area);
                        });
  }
}

template <bool W32>
__global__ void kc_hvel_scatter(GridGeom G, int64_t nb, const double *__restrict__ q,
                                const double *__restrict__ v, const uint8_t *__restrict__ fixed,
                                const double *__restrict__ m0, const double *__restrict__ w,
                                double *hmom, double *hmass) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= nb || fixed[b]) return;
  const double hl = G.h * 0.25;
  const double mass = m0[b] * w[b];
  const double vx = v[3 * b], vy = v[3 * b + 1];
  const double x = q[3 * b], y = q[3 * b + 1];
  int x0, y0, x1, y1;
  stencil64(G.basis, x, y, hl, G.gx, G.gy, G.h, x0, y0, x1, y1);
  stencil_weights<W32>(G, x, y, hl, x0, y0, x1, y1,
                      [&](int ix, int iy, double wt) {
                        if (!node_ok(G, ix, iy)) return;
                        const int64_t i = (int64_t)iy * (G.nx + 1) + ix;
                        atomicAdd(&hmom[2 * i], wt * mass * vx);
                        atomicAdd(&hmom[2 * i + 1], wt * mass * vy);
                        atomicAdd(&hmass[i], wt * mass);
                      });
}

__global__ void kc_hvel_finish(int64_t nn, const double *__restrict__ hmom,
                               const double *__restrict__ hmass, double *hvel) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  if (hmass[i] > 0.0) {
    hvel[2 * i] += hmom[2 * i] / hmass[i];
    hvel[2 * i + 1] += hmom[2 * i + 1] / hmass[i];
  }
}

inline int blocks_for(int64_t n, int t) { return (int)std::max<int64_t>(1, (n + t - 1) / t); }

} // namespace

hg_status hybrid_alloc(hg_hybrid *h) {
  const int64_t nn = (int64_t)(h->m->p.nx + 1) * (h->m->p.ny + 1);
  const int64_t nb = std::max<int64_t>(h->d->cap, 1);
  const int64_t big = std::max(nn, nb) + 1;
  hg_status st;
  if ((st = h->dem_mass.alloc(nn)) || (st = h->dem_mom.alloc(2 * nn)) ||
      (st = h->v_after.alloc(2 * nn)) || (st = h->a_after.alloc(2 * nn)) ||
      (st = h->pos_before.alloc(3 * nb)) || (st = h->hstress.alloc(4 * nn)) ||
      (st = h->hvel.alloc(2 * nn)) || (st = h->hmom.alloc(2 * nn)) ||
      (st = h->hmass.alloc(nn)) || (st = h->coupled.alloc(nb + 1)) ||
      (st = h->packed_dem.alloc(nb)) || (st = h->packed_mpm.alloc(nn)) ||
      (st = h->flag_tmp.alloc(big)) || (st = h->scan_tmp.alloc(scan_tmp_size(big))) ||
      (st = h->node_flag.alloc(nn + 1)) || (st = h->node_pos.alloc(nn + 1)) ||
      (st = h->counts.alloc(2)))
    return st;
  cudaStream_t s = h->ctx->stream;
  if (h->m->p.precision == HG_PRECISION_MIXED) {
    if ((st = h->homog.alloc(nn)) || (st = h->hl0.alloc(1))) return st;
    HG_LAUNCH(kc_set_scalar, 1, 1, 0, s, h->hl0.p, 0.0);
    HG_CHECK_LAUNCH();
    h->hl0_value = 0.0;
    HG_LAUNCH(kc_fill, blocks_for(nn, 256), 256, 0, s, h->homog.p, nn, 1.0);
    HG_CHECK_LAUNCH();
  }
  HG_CUDA_TRY(cudaMemsetAsync(h->counts.p, 0, 2 * sizeof(int32_t), s));
  HG_CUDA_TRY(cudaMemsetAsync(h->dem_mass.p, 0, sizeof(double) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(h->dem_mom.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(h->v_after.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(h->a_after.p, 0, sizeof(double) * 2 * nn, s));
  hg_status r = hybrid_clear_homogenized(h);
  if (r != HG_OK) return r;
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hybrid_pack_lists(hg_hybrid *h) {
  if (h->packed_valid) return HG_OK;
  cudaStream_t s = h->ctx->stream;
  const int64_t nn = (int64_t)(h->m->p.nx + 1) * (h->m->p.ny + 1), nb = h->step_bodies;
  hg_status st;
  // std::stable_partition of the grains (Coupling.cpp:113-127): kc_grain_mass
  // flagged them
  HG_CUDA_TRY(cudaMemsetAsync(h->coupled.p + nb, 0, sizeof(int32_t), s));
  if ((st = exclusive_scan_i32(h->coupled.p, h->flag_tmp.p, nb + 1, h->scan_tmp.p, s))) return st;
  HG_LAUNCH(kc_pack, blocks_for(nb + 1, 256), 256, 0, s, nb, h->coupled.p, h->flag_tmp.p,
            h->packed_dem.p, h->counts.p);
  HG_CHECK_LAUNCH();
  // and of the nodes with DEM mass
  HG_LAUNCH(kc_flag_nodes, blocks_for(nn, 256), 256, 0, s, nn, h->dem_mass.p, h->node_flag.p);
  HG_CHECK_LAUNCH();
  HG_CUDA_TRY(cudaMemsetAsync(h->node_flag.p + nn, 0, sizeof(int32_t), s));
  if ((st = exclusive_scan_i32(h->node_flag.p, h->node_pos.p, nn + 1, h->scan_tmp.p, s)))
    return st;
  HG_LAUNCH(kc_pack, blocks_for(nn + 1, 256), 256, 0, s, nn, h->node_flag.p, h->node_pos.p,
            h->packed_mpm.p, h->counts.p + 1);
  HG_CHECK_LAUNCH();
  h->packed_valid = true;
  return HG_OK;
}

hg_status hybrid_clear_homogenized(hg_hybrid *h) {
  const int64_t nn = (int64_t)(h->m->p.nx + 1) * (h->m->p.ny + 1);
  cudaStream_t s = h->ctx->stream;
  HG_CUDA_TRY(cudaMemsetAsync(h->hstress.p, 0, sizeof(double) * 4 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(h->hvel.p, 0, sizeof(double) * 2 * nn, s));
  return HG_OK;
}

namespace {

// W32: the stencil weights of the coupling kernels in FP32 (a MIXED bulk)
template <bool W32>
hg_status hybrid_step_impl(hg_hybrid *h, double dt, int flags) {
  hg_mpm *m = h->m;
  hg_dem *d = h->d;
  cudaStream_t s = h->ctx->stream;
  const GridGeom G = geom(m);
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  const int64_t nb = d->n;
  const int gs = h->ctx->num_sms * 4;
  hg_status st;
  // copyPrePositionsFull (Coupling.cpp:529-531)
  if (nb > 0)
    HG_CUDA_TRY(cudaMemcpyAsync(h->pos_before.p, d->q.p, sizeof(double) * 3 * nb,
                                cudaMemcpyDeviceToDevice, s));
  // A MIXED MPM object (FP32 bulk, FP64 positions) runs the same sequence on
  // its FP32 grid: its P2G for this step was done by the previous particle
  // launch (or the upload), its grid update and G2P are separate launches.
  const bool mixed = m->p.precision == HG_PRECISION_MIXED;
  const double *hl0 = m->hl.p;
  if (mixed) {
    if ((st = mixed_step_begin(m))) return st;
    // points.hl(0) in world units: the half-width of the first uploaded point
    const double v = m->p.basis == HG_BASIS_UGIMP ? (double)m->hl_cells * m->p.h : 0.0;
    if (v != h->hl0_value) {
      HG_LAUNCH(kc_set_scalar, 1, 1, 0, s, h->hl0.p, v);
      HG_CHECK_LAUNCH();
      h->hl0_value = v;
    }
    hl0 = h->hl0.p;
  } else if ((st = mpm64_phase0(m))) {
    return st;
  }
  // rasterizeGrainMass (pre-step positions, no partially filled cells)
  HG_CUDA_TRY(cudaMemsetAsync(h->dem_mass.p, 0, sizeof(double) * nn, s));
  if (!mixed) HG_CUDA_TRY(cudaMemsetAsync(m->g_hyb.p, 0, sizeof(int32_t) * nn, s));
  if (nb > 0) {
    if (mixed)
      HG_LAUNCH(kc_grain_mass<float>, blocks_for(nb, 128), 128, 0, s, G, nb, h->pos_before.p,
                hl0, d->fixed.p, d->m0.p, d->w.p, (const float *)m->accm.p, h->dem_mass.p,
                h->coupled.p);
    else
      HG_LAUNCH(kc_grain_mass<double>, blocks_for(nb, 128), 128, 0, s, G, nb, h->pos_before.p,
                hl0, d->fixed.p, d->m0.p, d->w.p, (const double *)m->g_mass.p, h->dem_mass.p,
                h->coupled.p);
    HG_CHECK_LAUNCH();
  }
  // The coupled grains (flagged by kc_grain_mass) and nodes (DEM mass > 0)
  // are walked in place: each is handled on its own and the scatters use
  // atomics, so the reference's packed order (Coupling.cpp:113-127) matters
  // only to callers of the lists, which hybrid_pack_lists builds on demand.
  h->packed_valid = false;
  h->step_bodies = nb;
  // DiscreteIntegrator::step -> flowWithWeight (DiscreteIntegrator.cpp:99-116)
  if ((st = dem_step(d, dt, 1))) return st;
  if ((st = mixed ? mixed_grid_update(m, dt) : mpm64_phase1(m, dt))) return st;
  // rasterizeGrainMom
  HG_CUDA_TRY(cudaMemsetAsync(h->dem_mom.p, 0, sizeof(double) * 2 * nn, s));
  HG_LAUNCH(kc_grain_mom<W32>, blocks_for(nb, 128), 128, 0, s, G, nb, h->coupled.p,
            h->pos_before.p, hl0, d->fixed.p, d->m0.p, d->w.p, d->v.p, h->dem_mom.p);
  HG_CHECK_LAUNCH();
  // updateVelocitiesOnGrid and the homogenisation factors
  if (mixed) {
    HG_LAUNCH(kc_update_nodes_x, blocks_for(nn, 256), 256, 0, s, nn, (const float *)m->gm.p,
              h->dem_mass.p, h->dem_mom.p, dt, m->va.p, h->v_after.p, h->a_after.p,
              h->homog.p);
  } else {
    HG_LAUNCH(kc_update_nodes, blocks_for(nn, 256), 256, 0, s, nn, m->g_mass.p, h->dem_mass.p,
              h->dem_mom.p, m->g_mom_new.p, h->v_after.p, h->a_after.p, m->g_homog.p);
  }
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kc_transfer<W32>, blocks_for(nb, 128), 128, 0, s, G, nb, h->coupled.p,
            h->pos_before.p, hl0, d->fixed.p, h->v_after.p, h->a_after.p, dt, d->v.p, d->q.p);
  HG_CHECK_LAUNCH();
  if ((st = mixed ? mixed_particles(m, dt) : mpm64_phase2(m, dt))) return st;
  if ((flags & HG_HYBRID_HOMOGENIZE_STRESS) && nb > 0) {
    HG_LAUNCH(kc_hstress<W32>, gs, 128, 0, s, G, nb, d->per_body_off.p, d->crec[d->cc].p, d->q.p,
              h->hstress.p);
    HG_CHECK_LAUNCH();
  }
  if ((flags & HG_HYBRID_HOMOGENIZE_VELOCITY) && nb > 0) {
    HG_CUDA_TRY(cudaMemsetAsync(h->hmom.p, 0, sizeof(double) * 2 * nn, s));
    HG_CUDA_TRY(cudaMemsetAsync(h->hmass.p, 0, sizeof(double) * nn, s));
    HG_LAUNCH(kc_hvel_scatter<W32>, blocks_for(nb, 128), 128, 0, s, G, nb, d->q.p, d->v.p,
              d->fixed.p, d->m0.p, d->w.p, h->hmom.p, h->hmass.p);
    HG_CHECK_LAUNCH();
    HG_LAUNCH(kc_hvel_finish, blocks_for(nn, 256), 256, 0, s, nn, h->hmom.p, h->hmass.p,
              h->hvel.p);
    HG_CHECK_LAUNCH();
  }
  return HG_OK;
}

} // namespace

hg_status hybrid_step(hg_hybrid *h, double dt, int flags) {
  return h->m->p.precision == HG_PRECISION_MIXED ? hybrid_step_impl<true>(h, dt, flags)
                                                 : hybrid_step_impl<false>(h, dt, flags);
}

} // namespace hg
