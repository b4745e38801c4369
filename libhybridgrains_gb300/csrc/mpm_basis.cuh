// FP64 MPM basis functions (linear and uGIMP linear), device and host, with the
// reference's operation order. Included by translation units compiled with
// --fmad=false.
#pragma once

namespace hg {

// LinearBasisFunctions.cpp:6-13
__host__ __device__ __forceinline__ double linear_n(double x) {
  const double a = fabs(x);
  return a < 1.0 ? 1.0 - a : 0.0;
}
// LinearBasisFunctions.cpp:16-22
__host__ __device__ __forceinline__ double linear_dn(double x) {
  if (fabs(x) <= 1.0) return (x >= 0.0) ? -1.0 : 1.0;
  return 0.0;
}
// uGIMPLinearBasisFunctions.cpp:6-22
__host__ __device__ __forceinline__ double lin_integral(double xp, double hl, double xi,
                                               double w) {
  const double diff = fabs(xp - xi);
  if (diff >= w + hl) return 0.0;
  if (diff >= w - hl) return (w + hl - diff) * (w + hl - diff) / (2.0 * w);
  if (diff >= hl) return 2.0 * hl * (1.0 - diff / w);
  return 2.0 * hl - (hl * hl + diff * diff) / w;
}
// uGIMPLinearBasisFunctions.cpp:24-42
__host__ __device__ __forceinline__ double lin_integral_grad(double xp, double hl,
                                                    double xi, double w) {
  const double diff = fabs(xp - xi);
  const double sgn = (xp - xi) >= 0.0 ? 1.0 : -1.0;
  if (diff >= w + hl) return 0.0;
  if (diff >= w - hl) return -sgn * (w + hl - diff) / w;
  if (diff >= hl) return -sgn * 2.0 * hl / w;
  return 2.0 * (xi - xp) / w;
}

// LinearBasisFunctions.cpp:49-62 / uGIMPLinearBasisFunctions.cpp:71-94.
// Inclusive node range; negative or too-large values mean out of grid.
__host__ __device__ __forceinline__ void stencil64(int basis, double x, double y,
                                          double hl, double gx, double gy,
                                          double h, int &x0, int &y0, int &x1,
                                          int &y1) {
  if (basis == HG_BASIS_LINEAR) {
    x0 = (int)floor((x - gx) / h);
    y0 = (int)floor((y - gy) / h);
    x1 = x0 + 1;
    y1 = y0 + 1;
  } else {
    x0 = (int)floor(((x - hl) - gx) / h);
    y0 = (int)floor(((y - hl) - gy) / h);
    x1 = (int)ceil(((x + hl) - gx) / h);
    y1 = (int)ceil(((y + hl) - gy) / h);
  }
}

// LinearBasisFunctions.cpp:81-97 / uGIMPLinearBasisFunctions.cpp:110-123
__host__ __device__ __forceinline__ double weight64(int basis, double x, double y,
                                           double hl, int ix, int iy, double gx,
                                           double gy, double h) {
  if (basis == HG_BASIS_LINEAR) {
    const double dx = ((x - h * (double)ix) - gx) / h;
    const double dy = ((y - h * (double)iy) - gy) / h;
    return linear_n(dx) * linear_n(dy);
  }
  const double xix = h * (double)ix + gx;
  const double xiy = h * (double)iy + gy;
  const double Vp = 4.0 * hl * hl;
  return lin_integral(x, hl, xix, h) * lin_integral(y, hl, xiy, h) / Vp;
}

// LinearBasisFunctions.cpp:115-136 / uGIMPLinearBasisFunctions.cpp:139-156
__host__ __device__ __forceinline__ void weight_grad64(int basis, double x, double y,
                                              double hl, int ix, int iy,
                                              double gx, double gy, double h,
                                              double &ox, double &oy) {
  if (basis == HG_BASIS_LINEAR) {
    const double dx = ((x - h * (double)ix) - gx) / h;
    const double dy = ((y - h * (double)iy) - gy) / h;
    const double wx = linear_n(dx), wy = linear_n(dy);
    ox = (wy * linear_dn(dx)) / h;
    oy = (wx * linear_dn(dy)) / h;
    return;
  }
  const double xix = h * (double)ix + gx;
  const double xiy = h * (double)iy + gy;
  const double Vp = 4.0 * hl * hl;
  const double wx = lin_integral(x, hl, xix, h);
  const double wy = lin_integral(y, hl, xiy, h);
  ox = wy * lin_integral_grad(x, hl, xix, h) / Vp;
  oy = wx * lin_integral_grad(y, hl, xiy, h) / Vp;
}

// Per-axis factors over a stencil of at most STENCIL_AXIS nodes from i0: a
// is the 1-D weight and b its derivative factor (linear: N(d) and dN(d) of
// d = ((x - h i) - g) / h; uGIMP: lin_integral and lin_integral_grad at
// x_i = h i + g). The 2-D weight and gradient are products of these in the
// order weight64 and weight_grad64 use, so they come out bit for bit the same
// while each 1-D factor is evaluated once per axis instead of once per node.
constexpr int STENCIL_AXIS = 4;

__host__ __device__ __forceinline__ void axis_factors(int basis, double x, double hl, int i0,
                                                      int count, double g, double h,
                                                      double a[STENCIL_AXIS],
                                                      double b[STENCIL_AXIS]) {
#pragma unroll
  for (int k = 0; k < STENCIL_AXIS; ++k) {
    a[k] = 0.0;
    b[k] = 0.0;
    if (k >= count) continue;
    const int i = i0 + k;
    if (basis == HG_BASIS_LINEAR) {
      const double d = ((x - h * (double)i) - g) / h;
      a[k] = linear_n(d);
      b[k] = linear_dn(d);
    } else {
      const double xi = h * (double)i + g;
      a[k] = lin_integral(x, hl, xi, h);
      b[k] = lin_integral_grad(x, hl, xi, h);
    }
  }
}

// The 1-D weights alone (the a of axis_factors).
__host__ __device__ __forceinline__ void axis_weights(int basis, double x, double hl, int i0,
                                                      int count, double g, double h,
                                                      double a[STENCIL_AXIS]) {
#pragma unroll
  for (int k = 0; k < STENCIL_AXIS; ++k) {
    a[k] = 0.0;
    if (k >= count) continue;
    const int i = i0 + k;
    if (basis == HG_BASIS_LINEAR) {
      a[k] = linear_n(((x - h * (double)i) - g) / h);
    } else {
      a[k] = lin_integral(x, hl, h * (double)i + g, h);
    }
  }
}

// weight64 from the axis factors
__host__ __device__ __forceinline__ double weight_ax(int basis, double ax, double ay, double hl) {
  if (basis == HG_BASIS_LINEAR) return ax * ay;
  const double Vp = 4.0 * hl * hl;
  return ax * ay / Vp;
}

// weight_grad64 from the axis factors
__host__ __device__ __forceinline__ void grad_ax(int basis, double ax, double bx, double ay,
                                                 double by, double hl, double h, double &ox,
                                                 double &oy) {
  if (basis == HG_BASIS_LINEAR) {
    ox = (ay * bx) / h;
    oy = (ax * by) / h;
    return;
  }
  const double Vp = 4.0 * hl * hl;
  ox = ay * bx / Vp;
  oy = ax * by / Vp;
}

// Visits the stencil's nodes in the reference's order (y outer, x inner) with
// weight64 of each, the 1-D factors evaluated once per axis when the stencil
// has at most STENCIL_AXIS nodes per axis.
template <class F>
__device__ __forceinline__ void for_stencil_weights(int basis, double x, double y, double hl,
                                                    int x0, int y0, int x1, int y1, double gx,
                                                    double gy, double h, F &&f) {
  const int nxs = x1 - x0 + 1, nys = y1 - y0 + 1;
  if (nxs <= STENCIL_AXIS && nys <= STENCIL_AXIS) {
    double ax[STENCIL_AXIS], ay[STENCIL_AXIS];
    axis_weights(basis, x, hl, x0, nxs, gx, h, ax);
    axis_weights(basis, y, hl, y0, nys, gy, h, ay);
#pragma unroll
    for (int ky = 0; ky < STENCIL_AXIS; ++ky) {
      if (ky >= nys) break;
#pragma unroll
      for (int kx = 0; kx < STENCIL_AXIS; ++kx) {
        if (kx >= nxs) break;
        f(x0 + kx, y0 + ky, weight_ax(basis, ax[kx], ay[ky], hl));
      }
    }
    return;
  }
  for (int iy = y0; iy <= y1; ++iy)
    for (int ix = x0; ix <= x1; ++ix) f(ix, iy, weight64(basis, x, y, hl, ix, iy, gx, gy, h));
}

// The same stencil's weights in FP32, for the mixed-precision hybrid step
// (its MPM bulk is FP32). The offset of the position from the stencil's
// first node, in cell widths, is formed in FP64 and rounded to FP32 once; the
// 1-D weights are those of LinearBasisFunctions.cpp:6-13 and
// uGIMPLinearBasisFunctions.cpp:6-22 in units of the cell width (for uGIMP,
// L(d) with a = hl / h: (1 + a - d)^2 / 2, 2a (1 - d) or 2a - (a^2 + d^2)
// by band, and the 2-D weight Lx Ly / (4 a^2)). The node range is the FP64
// stencil's, so the coupled nodes are the FP64 path's. Stencils wider than
// STENCIL_AXIS take the FP64 weights.
__device__ __forceinline__ float weight1d32(int basis, float d, float a) {
  const float dd = fabsf(d);
  if (basis == HG_BASIS_LINEAR) return dd < 1.0f ? 1.0f - dd : 0.0f;
  if (dd >= 1.0f + a) return 0.0f;
  if (dd >= 1.0f - a) return 0.5f * (1.0f + a - dd) * (1.0f + a - dd);
  if (dd >= a) return 2.0f * a * (1.0f - dd);
  return 2.0f * a - (a * a + dd * dd);
}
template <class F>
__device__ __forceinline__ void for_stencil_weights32(int basis, double x, double y, double hl,
                                                      int x0, int y0, int x1, int y1, double gx,
                                                      double gy, double h, double inv_h, F &&f) {
  const int nxs = x1 - x0 + 1, nys = y1 - y0 + 1;
  if (nxs > STENCIL_AXIS || nys > STENCIL_AXIS) {
    for_stencil_weights(basis, x, y, hl, x0, y0, x1, y1, gx, gy, h, f);
    return;
  }
  const float ox = (float)((x - gx) * inv_h - (double)x0);
  const float oy = (float)((y - gy) * inv_h - (double)y0);
  const float a = (float)(hl * inv_h);
  const float norm = basis == HG_BASIS_LINEAR ? 1.0f : 1.0f / (4.0f * a * a);
  float ax[STENCIL_AXIS], ay[STENCIL_AXIS];
#pragma unroll
  for (int k = 0; k < STENCIL_AXIS; ++k) {
    ax[k] = k < nxs ? weight1d32(basis, ox - (float)k, a) : 0.0f;
    ay[k] = k < nys ? weight1d32(basis, oy - (float)k, a) * norm : 0.0f;
  }
#pragma unroll
  for (int ky = 0; ky < STENCIL_AXIS; ++ky) {
    if (ky >= nys) break;
#pragma unroll
    for (int kx = 0; kx < STENCIL_AXIS; ++kx) {
      if (kx >= nxs) break;
      f(x0 + kx, y0 + ky, (double)(ax[kx] * ay[ky]));
    }
  }
}

} // namespace hg
