// CPU oracle: explicit MPM step of mpmgrains2d, restated in plain C++ (FP64).
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). Each function names the
// reference file:line it restates. The serial branches of the reference
// (the `#ifndef OPENMP_ENABLED` code) fix the summation order used when
// nthreads == 1; nthreads > 1 reproduces the reference's OpenMP scheme
// (per-thread full-grid scratch copies reduced node-wise,
// mpmgrains2d/PhysicsGrid.cpp:214-265) and is what bench.py times as the
// CPU baseline.
#include "oracle_state.h"

#include <algorithm>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace hgo {

// ---- basis functions -------------------------------------------------------

// LinearBasisFunctions.cpp:6-13
inline double linearN(double x) {
  const double a = std::fabs(x);
  return a < 1.0 ? 1.0 - a : 0.0;
}
// LinearBasisFunctions.cpp:16-22
inline double lineardN(double x) {
  if (std::fabs(x) <= 1.0) return (x >= 0.0) ? -1.0 : 1.0;
  return 0.0;
}
// uGIMPLinearBasisFunctions.cpp:6-22
inline double linIntegral(double xp, double hl, double xi, double w) {
  const double diff = std::fabs(xp - xi);
  if (diff >= w + hl) return 0.0;
  if (diff >= w - hl) return (w + hl - diff) * (w + hl - diff) / (2.0 * w);
  if (diff >= hl) return 2.0 * hl * (1.0 - diff / w);
  return 2.0 * hl - (hl * hl + diff * diff) / w;
}
// uGIMPLinearBasisFunctions.cpp:24-42
inline double linIntegralGrad(double xp, double hl, double xi, double w) {
  const double diff = std::fabs(xp - xi);
  const double sgn = (xp - xi) >= 0.0 ? 1.0 : -1.0;
  if (diff >= w + hl) return 0.0;
  if (diff >= w - hl) return -sgn * (w + hl - diff) / w;
  if (diff >= hl) return -sgn * 2.0 * hl / w;
  return 2.0 * (xi - xp) / w;
}

// LinearBasisFunctions.cpp:49-62 / uGIMPLinearBasisFunctions.cpp:71-94.
// The reference casts floor() to unsigned; an out-of-grid point wraps. The
// caller checks the range before indexing.
Stencil stencilOf(int basis, V2 x, double hl, V2 gmin, double h) {
  Stencil s;
  if (basis == LINEAR) {
    s.x0 = (unsigned)(long long)std::floor((x.x - gmin.x) / h);
    s.y0 = (unsigned)(long long)std::floor((x.y - gmin.y) / h);
    s.x1 = s.x0 + 1;
    s.y1 = s.y0 + 1;
  } else {
    s.x0 = (unsigned)(long long)std::floor(((x.x - hl) - gmin.x) / h);
    s.y0 = (unsigned)(long long)std::floor(((x.y - hl) - gmin.y) / h);
    s.x1 = (unsigned)(long long)std::ceil(((x.x + hl) - gmin.x) / h);
    s.y1 = (unsigned)(long long)std::ceil(((x.y + hl) - gmin.y) / h);
  }
  return s;
}

// LinearBasisFunctions.cpp:81-97 / uGIMPLinearBasisFunctions.cpp:110-123
double weightOf(int basis, V2 x, double hl, unsigned ix, unsigned iy,
                       V2 gmin, double h) {
  if (basis == LINEAR) {
    const double dx = ((x.x - h * (double)ix) - gmin.x) / h;
    const double dy = ((x.y - h * (double)iy) - gmin.y) / h;
    return linearN(dx) * linearN(dy);
  }
  const double xix = h * (double)ix + gmin.x;
  const double xiy = h * (double)iy + gmin.y;
  const double Vp = 4.0 * hl * hl;
  return linIntegral(x.x, hl, xix, h) * linIntegral(x.y, hl, xiy, h) / Vp;
}

// LinearBasisFunctions.cpp:115-136 / uGIMPLinearBasisFunctions.cpp:139-156
V2 weightGradOf(int basis, V2 x, double hl, unsigned ix, unsigned iy,
                       V2 gmin, double h) {
  if (basis == LINEAR) {
    const double dx = ((x.x - h * (double)ix) - gmin.x) / h;
    const double dy = ((x.y - h * (double)iy) - gmin.y) / h;
    const double wx = linearN(dx), wy = linearN(dy);
    V2 g{wy * lineardN(dx), wx * lineardN(dy)};
    g.x /= h;
    g.y /= h;
    return g;
  }
  const double xix = h * (double)ix + gmin.x;
  const double xiy = h * (double)iy + gmin.y;
  const double Vp = 4.0 * hl * hl;
  const double wx = linIntegral(x.x, hl, xix, h);
  const double wy = linIntegral(x.y, hl, xiy, h);
  return {wy * linIntegralGrad(x.x, hl, xix, h) / Vp,
          wx * linIntegralGrad(x.y, hl, xiy, h) / Vp};
}

inline bool nodeValid(const MpmState &s, unsigned ix, unsigned iy) {
  return ix <= s.nx && iy <= s.ny;
}

// ---- constitutive model (ConstitutiveModel.cpp) -----------------------------

// ConstitutiveModel.cpp:19-22
inline M2 elasticPrediction(M2 be_n, M2 L, double dt) {
  return madd(be_n, mscl(dt, madd(mmul(L, be_n), mmul(be_n, mT(L)))));
}

// ConstitutiveModel.cpp:26-81 (diagnostic prints omitted)
inline M2 plasticCorrection(M2 be_star, double kappa, double mu, double alpha,
                            int &jh) {
  if (jh != 0) {
    const double J = std::sqrt(mdet(be_star));
    if (J > 1.0) return mident(J);
    jh = 0;
  }
  const M2 b = be_star;
  const double J = std::sqrt(mdet(b));
  const double ys =
      std::max<double>(0.0, 0.5 * alpha * kappa * (1.0 + J) * (1.0 - J));
  const double half_tr = 0.5 * mtrace(b);
  const M2 dev = msub(b, mident(half_tr));
  const M2 bar_dev = mdiv(dev, J);
  if (mu * mnorm(bar_dev) > ys) {
    const double lambda2 = ys / (mu * mnorm(bar_dev));
    const double l1sq = mdet(b) - lambda2 * lambda2 * mdet(dev);
    const double lambda1 = std::sqrt(l1sq);
    return madd(mident(lambda1), mscl(lambda2, dev));
  }
  return b;
}

// ConstitutiveModel.cpp:83-97
inline M2 computeTau(M2 be, double kappa, double mu, int jh) {
  if (jh != 0) return M2{0, 0, 0, 0};
  const double J = std::sqrt(mdet(be));
  const M2 be_bar = mdiv(be, std::pow(mdet(be), 1.0 / 2.0));
  const double tr = mtrace(be_bar);
  const M2 dev = msub(be_bar, M2{tr / 2.0, 0.0, 0.0, tr / 2.0});
  const double s = kappa * 0.5 * (J + 1.0) * (J - 1.0);
  return madd(mident(s), mscl(mu, dev));
}

// MaterialPoints.cpp:290-294
inline M2 normalizedDeterminant(M2 A) {
  return mdiv(A, std::pow(mdet(A), 1.0 / 2.0));
}

// ---- grid ------------------------------------------------------------------

// PhysicsGrid.cpp:14-55
void setDimensions(MpmState &s, V2 gmin, V2 gmax, double h) {
  const V2 center{0.5 * (gmin.x + gmax.x), 0.5 * (gmin.y + gmax.y)};
  V2 width{gmax.x - gmin.x, gmax.y - gmin.y};
  s.nx = (unsigned)std::ceil(width.x / h);
  s.ny = (unsigned)std::ceil(width.y / h);
  width = {(double)s.nx * h, (double)s.ny * h};
  s.gmin = {center.x - 0.5 * width.x, center.y - 0.5 * width.y};
  s.gmax = {center.x + 0.5 * width.x, center.y + 0.5 * width.y};
  s.h = h;
  const unsigned n = s.nnodes();
  s.mass.assign(n, 0.0);
  s.mom.assign(2 * n, 0.0);
  s.mom_new.assign(2 * n, 0.0);
  s.force.assign(2 * n, 0.0);
  s.vel.assign(2 * n, 0.0);
  s.acc.assign(2 * n, 0.0);
  s.coupling_force.assign(2 * n, 0.0);
  s.homog.assign(n, 1.0);
  // The reference only resizes `hybridized` (PhysicsGrid.cpp:54), leaving it
  // uninitialised outside hybrid runs; the coupling zeroes it
  // (hybridgrains2dnew/Coupling.cpp:38). Zero is the defined value here.
  s.hybridized.assign(n, 0);
}

// PhysicsGrid.cpp:107-114
void clearRasterizedData(MpmState &s) {
  std::fill(s.mass.begin(), s.mass.end(), 0.0);
  std::fill(s.mom.begin(), s.mom.end(), 0.0);
  std::fill(s.mom_new.begin(), s.mom_new.end(), 0.0);
  std::fill(s.force.begin(), s.force.end(), 0.0);
  std::fill(s.vel.begin(), s.vel.end(), 0.0);
  std::fill(s.acc.begin(), s.acc.end(), 0.0);
}

inline int threadsFor(const MpmState &s) {
#ifdef _OPENMP
  return s.nthreads > 1 ? s.nthreads : 1;
#else
  (void)s;
  return 1;
#endif
}

// Scatter helper: serial order when one thread (PhysicsGrid.cpp:171-210,
// 277-330, 416-471); otherwise per-thread full-grid copies reduced node-wise
// in thread order (PhysicsGrid.cpp:214-265, 337-392, 477-542).
template <int NC, typename F>
void scatterParticles(MpmState &s, std::vector<double> &dst, F &&contrib) {
  const int T = threadsFor(s);
  if (T == 1) {
    for (int p = 0; p < s.np; ++p) contrib(p, dst.data());
    return;
  }
#ifdef _OPENMP
  static std::vector<std::vector<double>> scratch;
  if ((int)scratch.size() != T) scratch.assign(T, {});
#pragma omp parallel for num_threads(T)
  for (int t = 0; t < T; ++t) scratch[t].assign(dst.size(), 0.0);
#pragma omp parallel for num_threads(T) schedule(static)
  for (int p = 0; p < s.np; ++p) contrib(p, scratch[omp_get_thread_num()].data());
  const long n = (long)dst.size() / NC;
#pragma omp parallel for num_threads(T) schedule(static)
  for (long i = 0; i < n; ++i)
    for (int t = 0; t < T; ++t)
      for (int c = 0; c < NC; ++c) dst[NC * i + c] += scratch[t][NC * i + c];
#endif
}

// PhysicsGrid.cpp:168-272
void rasterizePointMasses(MpmState &s) {
  scatterParticles<1>(s, s.mass, [&](int p, double *mass) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        mass[s.flat(ix, iy)] += w * s.m[p];
      }
  });
}

// PhysicsGrid.cpp:274-411
void rasterizePointMomentum(MpmState &s) {
  scatterParticles<2>(s, s.mom, [&](int p, double *mom) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    const V2 pm{s.m[p] * s.v[2 * p], s.m[p] * s.v[2 * p + 1]};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        const unsigned i = s.flat(ix, iy);
        mom[2 * i] += w * pm.x;
        mom[2 * i + 1] += w * pm.y;
      }
  });
}

// MaterialPoints.cpp:183-202
void computeHyperelasticCauchyStress(MpmState &s) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    M2 tau{0, 0, 0, 0};
    if (s.J[p] <= 1.0)
      tau = computeTau(mscl(s.J[p], s.bep(p)), s.kappa, s.mu, s.jh[p]);
    const M2 sg = mdiv(tau, s.J[p]);
    s.sigma[4 * p] = sg.a00;
    s.sigma[4 * p + 1] = sg.a10;
    s.sigma[4 * p + 2] = sg.a01;
    s.sigma[4 * p + 3] = sg.a11;
  }
}

// PhysicsGrid.cpp:413-563
void computeForces(MpmState &s) {
  scatterParticles<2>(s, s.force, [&](int p, double *force) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    const M2 sg = s.sigp(p);
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        if (w == 0.0) continue;
        const V2 wg = weightGradOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        const double c = -s.vol[p] * s.J[p];
        const V2 sw = mvec(sg, wg);
        const unsigned i = s.flat(ix, iy);
        force[2 * i] += c * sw.x;
        force[2 * i + 1] += c * sw.y;
      }
  });
  const unsigned n = s.nnodes();
  for (unsigned i = 0; i < n; ++i) {
    if (s.hybridized[i] > 0) {
      s.force[2 * i] += 0.5 * s.mass[i] * s.g.x;
      s.force[2 * i + 1] += 0.5 * s.mass[i] * s.g.y;
    } else {
      s.force[2 * i] += s.mass[i] * s.g.x;
      s.force[2 * i + 1] += s.mass[i] * s.g.y;
    }
  }
  for (unsigned i = 0; i < 2 * n; ++i) s.force[i] += s.coupling_force[i];
}

// PhysicsGrid.cpp:565-586
void updateMomentum(MpmState &s, double dt) {
  const unsigned n = s.nnodes();
  for (unsigned i = 0; i < n; ++i)
    if (s.mass[i] > 0.0) {
      s.mom_new[2 * i] = s.mom[2 * i] + dt * s.force[2 * i];
      s.mom_new[2 * i + 1] = s.mom[2 * i + 1] + dt * s.force[2 * i + 1];
    }
}

// PhysicsGrid.cpp:611-673
void resolveGridPlaneCollisions(MpmState &s) {
  const unsigned n = s.nnodes();
  for (unsigned i = 0; i < n; ++i) {
    const unsigned ix = i % (s.nx + 1), iy = i / (s.nx + 1);
    const V2 px{s.gmin.x + s.h * (double)ix, s.gmin.y + s.h * (double)iy};
    for (const MpmPlane &pl : s.planes) {
      if (px.y < pl.lower_bound) continue;
      const double d = dot(pl.n, sub(px, pl.x));
      if (d > 0.0) continue;
      if (!pl.sticking) {
        if (s.mass[i] <= 0.0) continue;
        V2 vel{s.mom_new[2 * i] / s.mass[i], s.mom_new[2 * i + 1] / s.mass[i]};
        const double vn = dot(pl.n, vel);
        if (vn > 0.0) continue;
        vel = sub(vel, scl(vn, pl.n));
        s.mom_new[2 * i] = s.mass[i] * vel.x;
        s.mom_new[2 * i + 1] = s.mass[i] * vel.y;
      } else {
        s.mom_new[2 * i] = 0.0;
        s.mom_new[2 * i + 1] = 0.0;
      }
    }
  }
}

// PhysicsGrid.cpp:588-609
void lumpedMassVelocityAndAccelerationUpdate(MpmState &s, double dt) {
  const unsigned n = s.nnodes();
  for (unsigned i = 0; i < n; ++i) {
    if (s.mass[i] > 0.0) {
      s.vel[2 * i] = s.mom_new[2 * i] / s.mass[i];
      s.vel[2 * i + 1] = s.mom_new[2 * i + 1] / s.mass[i];
      const double dm = dt * s.mass[i];
      s.acc[2 * i] = (s.mom_new[2 * i] - s.mom[2 * i]) / dm;
      s.acc[2 * i + 1] = (s.mom_new[2 * i + 1] - s.mom[2 * i + 1]) / dm;
    } else {
      s.vel[2 * i] = s.vel[2 * i + 1] = 0.0;
      s.acc[2 * i] = s.acc[2 * i + 1] = 0.0;
    }
  }
}

// MaterialPoints.cpp:296-322
void computeVelGrad(MpmState &s) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    M2 L{0, 0, 0, 0};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const V2 gw = weightGradOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        const unsigned i = s.flat(ix, iy);
        const V2 vv{s.vel[2 * i], s.vel[2 * i + 1]};
        // grad_v += v * gw^T
        L = madd(L, M2{vv.x * gw.x, vv.y * gw.x, vv.x * gw.y, vv.y * gw.y});
      }
    s.velgrad[4 * p] = L.a00;
    s.velgrad[4 * p + 1] = L.a10;
    s.velgrad[4 * p + 2] = L.a01;
    s.velgrad[4 * p + 3] = L.a11;
  }
}

// MaterialPoints.cpp:324-348
void elasticPredictionPass(MpmState &s, double dt) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    const M2 L{s.velgrad[4 * p], s.velgrad[4 * p + 1], s.velgrad[4 * p + 2],
               s.velgrad[4 * p + 3]};
    const M2 bs = elasticPrediction(mscl(s.J[p], s.bep(p)), L, dt);
    s.J[p] = std::sqrt(mdet(bs));
    s.setbe(p, normalizedDeterminant(bs));
  }
}

// MaterialPoints.cpp:350-369
void plasticCorrectionPass(MpmState &s) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    const M2 bn = plasticCorrection(mscl(s.J[p], s.bep(p)), s.kappa, s.mu,
                                    s.dp_alpha, s.jh[p]);
    s.J[p] = std::sqrt(mdet(bn));
    s.setbe(p, normalizedDeterminant(bn));
  }
}

// MaterialPoints.cpp:204-245
void updateVelocities(MpmState &s, double dt) {
  const int T = threadsFor(s);
  const double a = s.flip_alpha;
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    V2 vpic{0, 0}, accel{0, 0};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        const unsigned i = s.flat(ix, iy);
        vpic = add(vpic, scl(w, V2{s.vel[2 * i], s.vel[2 * i + 1]}));
        accel = add(accel, scl(w, V2{s.acc[2 * i], s.acc[2 * i + 1]}));
      }
    const V2 vflip{s.v[2 * p] + accel.x * dt, s.v[2 * p + 1] + accel.y * dt};
    if (!s.kin[p]) {
      s.v[2 * p] = (1.0 - a) * vpic.x + a * vflip.x;
      s.v[2 * p + 1] = (1.0 - a) * vpic.y + a * vflip.y;
    }
  }
}

// MaterialPoints.cpp:247-288
void updatePositions(MpmState &s, double dt) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    const V2 x = s.qp(p);
    const Stencil st = stencilOf(s.basis, x, s.hl[p], s.gmin, s.h);
    V2 gv{0, 0};
    for (unsigned iy = st.y0; iy <= st.y1; ++iy)
      for (unsigned ix = st.x0; ix <= st.x1; ++ix) {
        const double w = weightOf(s.basis, x, s.hl[p], ix, iy, s.gmin, s.h);
        const unsigned i = s.flat(ix, iy);
        gv = add(gv, scl(w, V2{s.vel[2 * i], s.vel[2 * i + 1]}));
      }
    if (!s.kin[p]) {
      s.q[2 * p] += dt * gv.x;
      s.q[2 * p + 1] += dt * gv.y;
    } else {
      s.q[2 * p] += dt * s.v[2 * p];
      s.q[2 * p + 1] += dt * s.v[2 * p + 1];
    }
  }
}

// MaterialPoints.cpp:371-423
void resolveParticlePlaneCollisions(MpmState &s) {
  const int T = threadsFor(s);
#pragma omp parallel for num_threads(T) if (T > 1)
  for (int p = 0; p < s.np; ++p) {
    for (const MpmPlane &pl : s.planes) {
      if (s.q[2 * p + 1] < pl.lower_bound) continue;
      const double d = dot(pl.n, sub(s.qp(p), pl.x));
      if (d > 0.0) continue;
      s.q[2 * p] += -d * pl.n.x;
      s.q[2 * p + 1] += -d * pl.n.y;
      if (!pl.sticking) {
        const V2 vv{s.v[2 * p], s.v[2 * p + 1]};
        const double vn = dot(pl.n, vv);
        if (vn > 0.0) continue;
        s.v[2 * p] = vv.x - vn * pl.n.x;
        s.v[2 * p + 1] = vv.y - vn * pl.n.y;
      } else {
        s.v[2 * p] = 0.0;
        s.v[2 * p + 1] = 0.0;
      }
    }
  }
}

// ExplicitIntegrator.cpp:5-16
void mpmPhase0(MpmState &s) {
  clearRasterizedData(s);
  rasterizePointMasses(s);
  rasterizePointMomentum(s);
}
// ExplicitIntegrator.cpp:18-34
void mpmPhase1(MpmState &s, double dt) {
  computeHyperelasticCauchyStress(s);
  computeForces(s);
  updateMomentum(s, dt);
  resolveGridPlaneCollisions(s);
}
// ExplicitIntegrator.cpp:36-61
void mpmPhase2(MpmState &s, double dt) {
  lumpedMassVelocityAndAccelerationUpdate(s, dt);
  computeVelGrad(s);
  elasticPredictionPass(s, dt);
  plasticCorrectionPass(s);
  updateVelocities(s, dt);
  updatePositions(s, dt);
  resolveParticlePlaneCollisions(s);
}

} // namespace hgo

using namespace hgo;

// ---- C interface used by tests/ and bench.py ------------------------------

extern "C" {

void *hgo_mpm_create(const double *gmin, const double *gmax, double h,
                     int basis, double shear_modulus, double bulk_modulus,
                     double dp_alpha, double flip_alpha, const double *g) {
  MpmState *s = new MpmState();
  setDimensions(*s, V2{gmin[0], gmin[1]}, V2{gmax[0], gmax[1]}, h);
  s->basis = basis;
  s->mu = shear_modulus;
  s->kappa = bulk_modulus;
  s->dp_alpha = dp_alpha;
  s->flip_alpha = flip_alpha;
  s->g = V2{g[0], g[1]};
  return s;
}

void hgo_mpm_destroy(void *h) { delete static_cast<MpmState *>(h); }

void hgo_mpm_set_threads(void *h, int n) {
  static_cast<MpmState *>(h)->nthreads = n;
}

void hgo_mpm_add_plane(void *h, const double *x, const double *n, int sticking,
                       double lower_bound) {
  MpmState &s = *static_cast<MpmState *>(h);
  // StaticPlane.cpp:6-12: the normal is normalised on construction.
  s.planes.push_back(MpmPlane{V2{x[0], x[1]}, normalized(V2{n[0], n[1]}),
                           sticking, lower_bound});
}

// Grid geometry after PhysicsGrid::setDimensions: gmin[2], gmax[2], nx, ny.
void hgo_mpm_grid_info(void *h, double *gmin, double *gmax, unsigned *nxny) {
  MpmState &s = *static_cast<MpmState *>(h);
  gmin[0] = s.gmin.x;
  gmin[1] = s.gmin.y;
  gmax[0] = s.gmax.x;
  gmax[1] = s.gmax.y;
  nxny[0] = s.nx;
  nxny[1] = s.ny;
}

// Particle arrays in the reference's layouts: q, v as 2xN column-major
// (x0 y0 x1 y1 ...), be_bar as N column-major 2x2 blocks.
void hgo_mpm_set_particles(void *h, int n, const double *q, const double *v,
                           const double *m, const double *vol,
                           const double *hl, const double *be,
                           const double *J, const int *jh,
                           const unsigned char *kin) {
  MpmState &s = *static_cast<MpmState *>(h);
  s.np = n;
  s.q.assign(q, q + 2 * n);
  s.v.assign(v, v + 2 * n);
  s.m.assign(m, m + n);
  s.vol.assign(vol, vol + n);
  s.hl.assign(hl, hl + n);
  s.be.assign(be, be + 4 * n);
  s.J.assign(J, J + n);
  s.jh.assign(jh, jh + n);
  s.kin.assign(kin, kin + n);
  s.sigma.assign(4 * n, 0.0);
  s.velgrad.assign(4 * n, 0.0);
}

void hgo_mpm_get_particles(void *h, double *q, double *v, double *be,
                           double *J, int *jh, double *sigma) {
  MpmState &s = *static_cast<MpmState *>(h);
  if (q) std::memcpy(q, s.q.data(), sizeof(double) * 2 * s.np);
  if (v) std::memcpy(v, s.v.data(), sizeof(double) * 2 * s.np);
  if (be) std::memcpy(be, s.be.data(), sizeof(double) * 4 * s.np);
  if (J) std::memcpy(J, s.J.data(), sizeof(double) * s.np);
  if (jh) std::memcpy(jh, s.jh.data(), sizeof(int) * s.np);
  if (sigma) std::memcpy(sigma, s.sigma.data(), sizeof(double) * 4 * s.np);
}

void hgo_mpm_get_grid(void *h, double *mass, double *mom, double *mom_new,
                      double *force, double *vel, double *acc) {
  MpmState &s = *static_cast<MpmState *>(h);
  const size_t n = s.nnodes();
  if (mass) std::memcpy(mass, s.mass.data(), sizeof(double) * n);
  if (mom) std::memcpy(mom, s.mom.data(), sizeof(double) * 2 * n);
  if (mom_new) std::memcpy(mom_new, s.mom_new.data(), sizeof(double) * 2 * n);
  if (force) std::memcpy(force, s.force.data(), sizeof(double) * 2 * n);
  if (vel) std::memcpy(vel, s.vel.data(), sizeof(double) * 2 * n);
  if (acc) std::memcpy(acc, s.acc.data(), sizeof(double) * 2 * n);
}

// Grid arrays the hybrid coupling writes between phases.
void hgo_mpm_set_grid_coupling(void *h, const int *hybridized,
                               const double *coupling_force) {
  MpmState &s = *static_cast<MpmState *>(h);
  const size_t n = s.nnodes();
  if (hybridized) s.hybridized.assign(hybridized, hybridized + n);
  if (coupling_force)
    s.coupling_force.assign(coupling_force, coupling_force + 2 * n);
}

void hgo_mpm_set_mom_new(void *h, const double *mom_new) {
  MpmState &s = *static_cast<MpmState *>(h);
  s.mom_new.assign(mom_new, mom_new + 2 * s.nnodes());
}

void hgo_mpm_phase0(void *h) { mpmPhase0(*static_cast<MpmState *>(h)); }
void hgo_mpm_phase1(void *h, double dt) {
  mpmPhase1(*static_cast<MpmState *>(h), dt);
}
void hgo_mpm_phase2(void *h, double dt) {
  mpmPhase2(*static_cast<MpmState *>(h), dt);
}
// ExplicitIntegrator::flow (ExplicitIntegrator.cpp:63-67), nsteps times.
void hgo_mpm_step(void *h, double dt, int nsteps) {
  MpmState &s = *static_cast<MpmState *>(h);
  for (int k = 0; k < nsteps; ++k) {
    mpmPhase0(s);
    mpmPhase1(s, dt);
    mpmPhase2(s, dt);
  }
}

// InitialSimulationState.cpp:48-145 (rasterizeRectangle). Writes at most
// `cap` points; returns the number generated (which may exceed cap).
int hgo_mpm_seed_rectangle(void *h, const double *rmin, const double *rmax,
                           double rho, int npd, const double *vel,
                           double omega, int cap, double *q, double *v,
                           double *m, double *vol, double *hl) {
  MpmState &s = *static_cast<MpmState *>(h);
  const unsigned bx0 = (unsigned)std::floor((rmin[0] - s.gmin.x) / s.h);
  const unsigned by0 = (unsigned)std::floor((rmin[1] - s.gmin.y) / s.h);
  const unsigned bx1 = (unsigned)std::ceil((rmax[0] - s.gmin.x) / s.h);
  const unsigned by1 = (unsigned)std::ceil((rmax[1] - s.gmin.y) / s.h);
  const V2 center{0.5 * (rmin[0] + rmax[0]), 0.5 * (rmin[1] + rmax[1])};
  const double half = 0.5 * s.h / (double)npd;
  const double pvol = half * half * 4.0;
  const double pmass = rho * pvol;
  int count = 0;
  for (unsigned gy = by0; gy < by1; ++gy)
    for (unsigned gx = bx0; gx < bx1; ++gx)
      for (int cy = 0; cy < npd; ++cy)
        for (int cx = 0; cx < npd; ++cx) {
          const V2 pos{
              s.gmin.x + s.h * ((double)gx + ((double)cx + 0.5) / (double)npd),
              s.gmin.y + s.h * ((double)gy + ((double)cy + 0.5) / (double)npd)};
          if (pos.x < rmin[0] || pos.y < rmin[1] || pos.x > rmax[0] ||
              pos.y > rmax[1])
            continue;
          // pointInsidePlane (InitialSimulationState.cpp:33-43)
          bool inside = false;
          for (const MpmPlane &pl : s.planes) {
            if (pos.y < pl.lower_bound) break;
            if (dot(pl.n, sub(pos, pl.x)) < 0.0) {
              inside = true;
              break;
            }
          }
          if (inside) continue;
          if (count < cap) {
            // v + omega * (z x arm): (-omega*arm.y, omega*arm.x)
            const V2 arm = sub(pos, center);
            q[2 * count] = pos.x;
            q[2 * count + 1] = pos.y;
            v[2 * count] = vel[0] + omega * (-arm.y);
            v[2 * count + 1] = vel[1] + omega * arm.x;
            m[count] = pmass;
            vol[count] = pvol;
            hl[count] = half;
          }
          ++count;
        }
  return count;
}

} // extern "C"
