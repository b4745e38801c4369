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

} // namespace hg
