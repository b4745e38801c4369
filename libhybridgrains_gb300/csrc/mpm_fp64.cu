// Plain FP64 MPM step: the drop-in for ExplicitIntegrator::flow with the
// reference's arithmetic in double precision.
//
// This translation unit is compiled with --fmad=false so that each multiply
// and add rounds separately, in the order the reference's Eigen expressions
// evaluate them (the CPU oracle is built the same way with
// -ffp-contract=off). Grid accumulation uses FP64 atomics, so node sums differ
// from the serial reference only in summation order.
//
// Kernels:
//   k64_p2g         rasterizePointMasses + rasterizePointMomentum
//                   (PhysicsGrid.cpp:168-411), computeHyperelasticCauchyStress
//                   (MaterialPoints.cpp:183-202) and the particle part of
//                   computeForces (PhysicsGrid.cpp:413-471)
//   k64_grid_phase1 node part of computeForces (PhysicsGrid.cpp:459-471),
//                   updateMomentum (565-586), resolvePlaneCollisions (611-673)
//   k64_grid_phase2 lumpedMassVelocityAndAccelerationUpdate (588-609)
//   k64_g2p         computeVelGrad, elasticPrediction, plasticCorrection,
//                   updateVelocities, updatePositions, resolvePlaneCollisions
//                   (MaterialPoints.cpp:204-423), fused per material point.
#include "hg_internal.cuh"
#include "mpm_basis.cuh"

namespace hg {

namespace {

struct M2d {
  double a00, a10, a01, a11;
};

__device__ __forceinline__ M2d m_add(M2d a, M2d b) {
  return {a.a00 + b.a00, a.a10 + b.a10, a.a01 + b.a01, a.a11 + b.a11};
}
__device__ __forceinline__ M2d m_sub(M2d a, M2d b) {
  return {a.a00 - b.a00, a.a10 - b.a10, a.a01 - b.a01, a.a11 - b.a11};
}
__device__ __forceinline__ M2d m_scl(double s, M2d a) {
  return {s * a.a00, s * a.a10, s * a.a01, s * a.a11};
}
__device__ __forceinline__ M2d m_div(M2d a, double s) {
  return {a.a00 / s, a.a10 / s, a.a01 / s, a.a11 / s};
}
__device__ __forceinline__ M2d m_mul(M2d a, M2d b) {
  return {a.a00 * b.a00 + a.a01 * b.a10, a.a10 * b.a00 + a.a11 * b.a10,
          a.a00 * b.a01 + a.a01 * b.a11, a.a10 * b.a01 + a.a11 * b.a11};
}
__device__ __forceinline__ M2d m_T(M2d a) { return {a.a00, a.a01, a.a10, a.a11}; }
__device__ __forceinline__ double m_det(M2d a) {
  return a.a00 * a.a11 - a.a10 * a.a01;
}
__device__ __forceinline__ double m_tr(M2d a) { return a.a00 + a.a11; }
__device__ __forceinline__ double m_norm(M2d a) {
  return sqrt(a.a00 * a.a00 + a.a10 * a.a10 + a.a01 * a.a01 + a.a11 * a.a11);
}
__device__ __forceinline__ M2d m_id(double s) { return {s, 0.0, 0.0, s}; }

__device__ __forceinline__ M2d load_m(const double *a, int64_t p) {
  return {a[4 * p], a[4 * p + 1], a[4 * p + 2], a[4 * p + 3]};
}
__device__ __forceinline__ void store_m(double *a, int64_t p, M2d m) {
  a[4 * p] = m.a00;
  a[4 * p + 1] = m.a10;
  a[4 * p + 2] = m.a01;
  a[4 * p + 3] = m.a11;
}

// ConstitutiveModel.cpp:83-97
__device__ M2d compute_tau(M2d be, double kappa, double mu, int jh) {
  if (jh != 0) return {0.0, 0.0, 0.0, 0.0};
  const double J = sqrt(m_det(be));
  const M2d be_bar = m_div(be, sqrt(m_det(be)));
  const double tr = m_tr(be_bar);
  const M2d dev = m_sub(be_bar, M2d{tr / 2.0, 0.0, 0.0, tr / 2.0});
  const double s = kappa * 0.5 * (J + 1.0) * (J - 1.0);
  return m_add(m_id(s), m_scl(mu, dev));
}

// ConstitutiveModel.cpp:26-81
__device__ M2d plastic_correction(M2d b, double kappa, double mu, double alpha,
                                  int &jh) {
  if (jh != 0) {
    const double J = sqrt(m_det(b));
    if (J > 1.0) return m_id(J);
    jh = 0;
  }
  const double J = sqrt(m_det(b));
  const double ys = fmax(0.0, 0.5 * alpha * kappa * (1.0 + J) * (1.0 - J));
  const double half_tr = 0.5 * m_tr(b);
  const M2d dev = m_sub(b, m_id(half_tr));
  const M2d bar_dev = m_div(dev, J);
  if (mu * m_norm(bar_dev) > ys) {
    const double lambda2 = ys / (mu * m_norm(bar_dev));
    const double l1sq = m_det(b) - lambda2 * lambda2 * m_det(dev);
    const double lambda1 = sqrt(l1sq);
    return m_add(m_id(lambda1), m_scl(lambda2, dev));
  }
  return b;
}

__device__ __forceinline__ bool finite2(double a, double b) {
  return isfinite(a) && isfinite(b);
}

__global__ void k64_p2g(MpmParams P, int64_t n, const double *__restrict__ q,
                        const double *__restrict__ v,
                        const double *__restrict__ m,
                        const double *__restrict__ vol,
                        const double *__restrict__ hl,
                        const double *__restrict__ be,
                        const double *__restrict__ J,
                        const int32_t *__restrict__ jh, double *sigma,
                        double *g_mass, double *g_mom, double *g_force,
                        uint32_t *status) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double x = q[2 * p], y = q[2 * p + 1];
  const double h = hl[p];
  int x0, y0, x1, y1;
  stencil64(P.basis, x, y, h, P.gmin[0], P.gmin[1], P.h, x0, y0, x1, y1);
  // Stress (MaterialPoints.cpp:183-202)
  M2d tau{0.0, 0.0, 0.0, 0.0};
  const double Jp = J[p];
  if (Jp <= 1.0) tau = compute_tau(m_scl(Jp, load_m(be, p)), P.kappa, P.mu, jh[p]);
  const M2d sg = m_div(tau, Jp);
  store_m(sigma, p, sg);
  if (x0 < 0 || y0 < 0 || x1 > P.nx || y1 > P.ny) {
    atomicOr(status, (uint32_t)HG_STATUS_OUT_OF_GRID);
    return;
  }
  const double mp = m[p];
  const double pmx = mp * v[2 * p], pmy = mp * v[2 * p + 1];
  const double c = -vol[p] * Jp;
  auto node = [&](int ix, int iy, double w, double gx, double gy) {
    const int64_t i = (int64_t)iy * (P.nx + 1) + ix;
    atomicAdd(&g_mass[i], w * mp);
    atomicAdd(&g_mom[2 * i], w * pmx);
    atomicAdd(&g_mom[2 * i + 1], w * pmy);
    if (w == 0.0) return;
    const double swx = sg.a00 * gx + sg.a01 * gy;
    const double swy = sg.a10 * gx + sg.a11 * gy;
    atomicAdd(&g_force[2 * i], c * swx);
    atomicAdd(&g_force[2 * i + 1], c * swy);
  };
  const int nxs = x1 - x0 + 1, nys = y1 - y0 + 1;
  if (nxs <= STENCIL_AXIS && nys <= STENCIL_AXIS) {
    double ax[STENCIL_AXIS], bx[STENCIL_AXIS], ay[STENCIL_AXIS], by[STENCIL_AXIS];
    axis_factors(P.basis, x, h, x0, nxs, P.gmin[0], P.h, ax, bx);
    axis_factors(P.basis, y, h, y0, nys, P.gmin[1], P.h, ay, by);
#pragma unroll
    for (int ky = 0; ky < STENCIL_AXIS; ++ky) {
      if (ky >= nys) break;
#pragma unroll
      for (int kx = 0; kx < STENCIL_AXIS; ++kx) {
        if (kx >= nxs) break;
        double gx, gy;
        grad_ax(P.basis, ax[kx], bx[kx], ay[ky], by[ky], h, P.h, gx, gy);
        node(x0 + kx, y0 + ky, weight_ax(P.basis, ax[kx], ay[ky], h), gx, gy);
      }
    }
    return;
  }
  for (int iy = y0; iy <= y1; ++iy)
    for (int ix = x0; ix <= x1; ++ix) {
      double gx, gy;
      weight_grad64(P.basis, x, y, h, ix, iy, P.gmin[0], P.gmin[1], P.h, gx, gy);
      node(ix, iy, weight64(P.basis, x, y, h, ix, iy, P.gmin[0], P.gmin[1], P.h), gx, gy);
    }
}

__global__ void k64_grid_phase1(MpmParams P, double dt,
                                const double *__restrict__ g_mass,
                                const double *__restrict__ g_mom,
                                double *g_mom_new, double *g_force,
                                const double *__restrict__ g_cforce,
                                const int32_t *__restrict__ g_hyb) {
  const int64_t nn = (int64_t)(P.nx + 1) * (P.ny + 1);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double mi = g_mass[i];
  double fx = g_force[2 * i], fy = g_force[2 * i + 1];
  if (g_hyb[i] > 0) {
    fx += 0.5 * mi * P.g[0];
    fy += 0.5 * mi * P.g[1];
  } else {
    fx += mi * P.g[0];
    fy += mi * P.g[1];
  }
  fx += g_cforce[2 * i];
  fy += g_cforce[2 * i + 1];
  g_force[2 * i] = fx;
  g_force[2 * i + 1] = fy;
  double pnx = g_mom_new[2 * i], pny = g_mom_new[2 * i + 1];
  if (mi > 0.0) {
    pnx = g_mom[2 * i] + dt * fx;
    pny = g_mom[2 * i + 1] + dt * fy;
  }
  // PhysicsGrid::resolvePlaneCollisions
  const int ix = (int)(i % (P.nx + 1)), iy = (int)(i / (P.nx + 1));
  const double px = P.gmin[0] + P.h * (double)ix;
  const double py = P.gmin[1] + P.h * (double)iy;
  for (int k = 0; k < P.nplanes; ++k) {
    const MpmPlaneDev &pl = P.planes[k];
    if (py < pl.lower_bound) continue;
    const double d = pl.n[0] * (px - pl.x[0]) + pl.n[1] * (py - pl.x[1]);
    if (d > 0.0) continue;
    if (!pl.sticking) {
      if (mi <= 0.0) continue;
      double vx = pnx / mi, vy = pny / mi;
      const double vn = pl.n[0] * vx + pl.n[1] * vy;
      if (vn > 0.0) continue;
      vx = vx - vn * pl.n[0];
      vy = vy - vn * pl.n[1];
      pnx = mi * vx;
      pny = mi * vy;
    } else {
      pnx = 0.0;
      pny = 0.0;
    }
  }
  g_mom_new[2 * i] = pnx;
  g_mom_new[2 * i + 1] = pny;
}

__global__ void k64_grid_phase2(MpmParams P, double dt,
                                const double *__restrict__ g_mass,
                                const double *__restrict__ g_mom,
                                const double *__restrict__ g_mom_new,
                                double *g_vel, double *g_acc) {
  const int64_t nn = (int64_t)(P.nx + 1) * (P.ny + 1);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double mi = g_mass[i];
  if (mi > 0.0) {
    g_vel[2 * i] = g_mom_new[2 * i] / mi;
    g_vel[2 * i + 1] = g_mom_new[2 * i + 1] / mi;
    const double dm = dt * mi;
    g_acc[2 * i] = (g_mom_new[2 * i] - g_mom[2 * i]) / dm;
    g_acc[2 * i + 1] = (g_mom_new[2 * i + 1] - g_mom[2 * i + 1]) / dm;
  } else {
    g_vel[2 * i] = 0.0;
    g_vel[2 * i + 1] = 0.0;
    g_acc[2 * i] = 0.0;
    g_acc[2 * i + 1] = 0.0;
  }
}

__global__ void k64_g2p(MpmParams P, double dt, int64_t n, double *q, double *v,
                        const double *__restrict__ hl, double *be, double *J,
                        int32_t *jh, const uint8_t *__restrict__ kin,
                        const double *__restrict__ g_vel,
                        const double *__restrict__ g_acc, uint32_t *status) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  double x = q[2 * p], y = q[2 * p + 1];
  const double h = hl[p];
  int x0, y0, x1, y1;
  stencil64(P.basis, x, y, h, P.gmin[0], P.gmin[1], P.h, x0, y0, x1, y1);
  if (x0 < 0 || y0 < 0 || x1 > P.nx || y1 > P.ny) {
    atomicOr(status, (uint32_t)HG_STATUS_OUT_OF_GRID);
    return;
  }
  const int64_t row = P.nx + 1;
  // axis factors of the start-of-step position (when the stencil fits)
  const int nxs = x1 - x0 + 1, nys = y1 - y0 + 1;
  const bool fits = nxs <= STENCIL_AXIS && nys <= STENCIL_AXIS;
  double ax[STENCIL_AXIS], bx[STENCIL_AXIS], ay[STENCIL_AXIS], by[STENCIL_AXIS];
  if (fits) {
    axis_factors(P.basis, x, h, x0, nxs, P.gmin[0], P.h, ax, bx);
    axis_factors(P.basis, y, h, y0, nys, P.gmin[1], P.h, ay, by);
  }
  // visits the stencil's nodes in the reference's order with their weight
  // and weight gradient
  auto each_node = [&](auto &&f) {
    if (fits) {
#pragma unroll
      for (int ky = 0; ky < STENCIL_AXIS; ++ky) {
        if (ky >= nys) break;
#pragma unroll
        for (int kx = 0; kx < STENCIL_AXIS; ++kx) {
          if (kx >= nxs) break;
          double gx, gy;
          grad_ax(P.basis, ax[kx], bx[kx], ay[ky], by[ky], h, P.h, gx, gy);
          f((int64_t)(y0 + ky) * row + (x0 + kx), weight_ax(P.basis, ax[kx], ay[ky], h), gx,
            gy);
        }
      }
      return;
    }
    for (int iy = y0; iy <= y1; ++iy)
      for (int ix = x0; ix <= x1; ++ix) {
        double gx, gy;
        weight_grad64(P.basis, x, y, h, ix, iy, P.gmin[0], P.gmin[1], P.h, gx, gy);
        f((int64_t)iy * row + ix, weight64(P.basis, x, y, h, ix, iy, P.gmin[0], P.gmin[1], P.h),
          gx, gy);
      }
  };
  // computeVelGrad (MaterialPoints.cpp:296-322)
  M2d L{0.0, 0.0, 0.0, 0.0};
  each_node([&](int64_t i, double, double gx, double gy) {
    const double vx = g_vel[2 * i], vy = g_vel[2 * i + 1];
    L = m_add(L, M2d{vx * gx, vy * gx, vx * gy, vy * gy});
  });
  // elasticPrediction (MaterialPoints.cpp:324-348, ConstitutiveModel.cpp:19-22)
  double Jp = J[p];
  M2d bb = load_m(be, p);
  {
    const M2d ben = m_scl(Jp, bb);
    const M2d bs = m_add(ben, m_scl(dt, m_add(m_mul(L, ben), m_mul(ben, m_T(L)))));
    Jp = sqrt(m_det(bs));
    bb = m_div(bs, sqrt(m_det(bs)));
  }
  // plasticCorrection (MaterialPoints.cpp:350-369)
  int jhp = jh[p];
  {
    const M2d bn = plastic_correction(m_scl(Jp, bb), P.kappa, P.mu, P.dp_alpha, jhp);
    Jp = sqrt(m_det(bn));
    bb = m_div(bn, sqrt(m_det(bn)));
  }
  // updateVelocities (MaterialPoints.cpp:204-245) and updatePositions
  // (247-288); both read the grid at the start-of-step position.
  double vpx = 0.0, vpy = 0.0, apx = 0.0, apy = 0.0, gvx = 0.0, gvy = 0.0;
  each_node([&](int64_t i, double w, double, double) {
    vpx = vpx + w * g_vel[2 * i];
    vpy = vpy + w * g_vel[2 * i + 1];
    apx = apx + w * g_acc[2 * i];
    apy = apy + w * g_acc[2 * i + 1];
  });
  gvx = vpx;
  gvy = vpy;
  double vx = v[2 * p], vy = v[2 * p + 1];
  const bool kinem = kin[p] != 0;
  if (!kinem) {
    const double a = P.flip_alpha;
    const double fx = vx + apx * dt, fy = vy + apy * dt;
    vx = (1.0 - a) * vpx + a * fx;
    vy = (1.0 - a) * vpy + a * fy;
    x += dt * gvx;
    y += dt * gvy;
  } else {
    x += dt * vx;
    y += dt * vy;
  }
  // MaterialPoints::resolvePlaneCollisions (MaterialPoints.cpp:371-423)
  for (int k = 0; k < P.nplanes; ++k) {
    const MpmPlaneDev &pl = P.planes[k];
    if (y < pl.lower_bound) continue;
    const double d = pl.n[0] * (x - pl.x[0]) + pl.n[1] * (y - pl.x[1]);
    if (d > 0.0) continue;
    x += -d * pl.n[0];
    y += -d * pl.n[1];
    if (!pl.sticking) {
      const double vn = pl.n[0] * vx + pl.n[1] * vy;
      if (vn > 0.0) continue;
      vx = vx - vn * pl.n[0];
      vy = vy - vn * pl.n[1];
    } else {
      vx = 0.0;
      vy = 0.0;
    }
  }
  if (!finite2(x, y) || !finite2(vx, vy) || !isfinite(Jp))
    atomicOr(status, (uint32_t)HG_STATUS_NONFINITE);
  q[2 * p] = x;
  q[2 * p + 1] = y;
  v[2 * p] = vx;
  v[2 * p + 1] = vy;
  store_m(be, p, bb);
  J[p] = Jp;
  jh[p] = jhp;
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

} // namespace

hg_status mpm64_phase0(hg_mpm *m) {
  cudaStream_t s = m->ctx->stream;
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  // clearRasterizedData (PhysicsGrid.cpp:107-114)
  HG_CUDA_TRY(cudaMemsetAsync(m->g_mass.p, 0, sizeof(double) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->g_mom.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->g_mom_new.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->g_force.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->g_vel.p, 0, sizeof(double) * 2 * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->g_acc.p, 0, sizeof(double) * 2 * nn, s));
  if (m->n > 0) {
    HG_LAUNCH(k64_p2g, blocks_for(m->n, 128), 128, 0, s, m->p, m->n, m->q.p,
              m->v.p, m->m.p, m->vol.p, m->hl.p, m->be.p, m->J.p, m->jh.p,
              m->sigma.p, m->g_mass.p, m->g_mom.p, m->g_force.p, m->status.p);
    HG_CHECK_LAUNCH();
  }
  return HG_OK;
}

hg_status mpm64_phase1(hg_mpm *m, double dt) {
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  HG_LAUNCH(k64_grid_phase1, blocks_for(nn, 256), 256, 0, m->ctx->stream, m->p,
            dt, m->g_mass.p, m->g_mom.p, m->g_mom_new.p, m->g_force.p,
            m->g_cforce.p, m->g_hyb.p);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

hg_status mpm64_phase2(hg_mpm *m, double dt) {
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  cudaStream_t s = m->ctx->stream;
  HG_LAUNCH(k64_grid_phase2, blocks_for(nn, 256), 256, 0, s, m->p, dt,
            m->g_mass.p, m->g_mom.p, m->g_mom_new.p, m->g_vel.p, m->g_acc.p);
  HG_CHECK_LAUNCH();
  if (m->n > 0) {
    HG_LAUNCH(k64_g2p, blocks_for(m->n, 128), 128, 0, s, m->p, dt, m->n, m->q.p,
              m->v.p, m->hl.p, m->be.p, m->J.p, m->jh.p, m->kin.p, m->g_vel.p,
              m->g_acc.p, m->status.p);
    HG_CHECK_LAUNCH();
  }
  return HG_OK;
}

} // namespace hg
