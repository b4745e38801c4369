// Mixed-precision MPM step (FP64 positions, FP32 everything else).
//
// One reference step (ExplicitIntegrator::flow, ExplicitIntegrator.cpp:63-67)
// is executed as two kernels:
//
//   kx_grid_update  node part of computeForces (gravity, coupling force),
//                   updateMomentum, PhysicsGrid::resolvePlaneCollisions and
//                   lumpedMassVelocityAndAccelerationUpdate
//                   (PhysicsGrid.cpp:459-673) over the active tiles only; it
//                   consumes the accumulated (m, p, f) and zeroes it.
//   kx_g2p2g        G2P of this step fused with P2G of the next one: per
//                   material point computeVelGrad, elasticPrediction,
//                   plasticCorrection, updateVelocities, updatePositions,
//                   resolvePlaneCollisions (MaterialPoints.cpp:204-423), then
//                   computeHyperelasticCauchyStress (183-202) at the new
//                   state and the rasterisation of mass, momentum and
//                   internal force (PhysicsGrid.cpp:168-471) for the next
//                   step. Each particle is read once and written once per
//                   step.
//
// Layout in HBM. Particles are SoA, sorted by (tile, cell within tile) with
// 16x16-cell tiles: u = (x - grid_min)/h as double2, v float2, (m, V) float2,
// strain float4 = (J - 1, be_bar - I [xx, xy, yy]), a flag byte and, with the
// uGIMP basis, the half-width in cells as a float. Storing
// J and be_bar as offsets from 1 and I keeps FP32's 24 bits on the strain
// itself rather than on the leading 1. Grid fields are dense node-major
// float4/float arrays; only tiles near particles are touched.
//
// P2G is cell-major: one thread per cell accumulates the contributions of the
// points sorted into its cell in registers (no atomics); points that left
// their cell since the last re-sort use shared-memory atomics on the tile's
// node window. Window sums go to global memory with one float4 + one float
// atomic per touched node. With the uGIMP basis (up to 3 x 3 nodes per point)
// one thread per point adds to the grid with global reductions.
//
// Re-sorting (counting sort by cell key) runs when a point has drifted out of
// its tile's window, when more than 1/32 of the points have left their sorted
// cell, and at least every MAX_STEPS_BETWEEN_REBINS steps. Points outside
// their window are still handled exactly (G2P from global velocity, P2G with
// global atomics), so the re-sort cadence affects speed only.
#include "hg_internal.cuh"
#include "scan_block.cuh"

#include <algorithm>
#include <array>
#include <chrono>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>

#include <cmath>

namespace hg {

namespace {

constexpr int THREADS = 256;
constexpr int MAX_BATCH = HG_MAX_BATCH; // scenes per batched launch

struct alignas(16) MixedArgs {
  int nx, ny, ntx, nty;
  int64_t n;
  double gmin[2], h; // grid origin and cell width (the node plane test)
  float dt, inv_h, kappa, mu, dp_alpha, flip_alpha, gx, gy;
  // Half-width (in cells) of the band around a plane in which the FP32
  // plane test is redone exactly in FP64.
  float pmargin;
  int nplanes;
  const int32_t *offsets;
  const int32_t *active;  // active bins or tiles
  const int32_t *nactive; // device count
  double2 *u;
  float2 *v;
  const float2 *mv;
  float4 *strain;
  uint8_t *flags;
  const float *hl; // uGIMP half-widths in cells (nullptr for the linear basis)
  const float4 *va;
  float4 *va_out; // the same array, written by the grid update
  float4 *acc4;
  float *accm;
  float *gm;
  uint32_t *status;
  uint32_t *outside;
  // last, so that a batched kernel copies only the nplanes planes in use
  MpmPlaneDev planes[HG_MAX_PLANES];
};

// Exact floor(u) and the fraction u - floor(u) truncated to 24 bits, using
// integer operations on the FP64 bit pattern (the FP64 pipe is ~1/64 of the
// FP32 rate on this part). Valid for 0 <= u < 2^23; other values take the
// FP64 path.
// Rare cases (u < 1, negative, huge or non-finite) are kept out of line so
// that the common path does not carry predicated FP64 instructions.
// Returned by value (cell, fraction bits): reference parameters would take
// the callers' variables' addresses and keep them in local memory on every
// path.
__device__ __noinline__ int2 split_u_slow(double u) {
  const double fl = floor(u);
  return make_int2((int)fl, __float_as_int(__double2float_rz(u - fl)));
}

__device__ __forceinline__ void split_u(double u, int &c, float &f) {
  // 32-bit word operations only: hi = sign | exponent | mantissa[51:32]
  const unsigned hi = (unsigned)__double2hiint(u), lo = (unsigned)__double2loint(u);
  const int e = (int)(hi >> 20) - 1023; // sign bit set gives e >= 1025
  if (e >= 0 && e < 23) {
    const unsigned hf = (hi & 0xFFFFFu) | 0x100000u; // 21 leading mantissa bits
    const int sh = 52 - e;                            // 30..52
    c = sh >= 32 ? (int)(hf >> (sh - 32)) : (int)__funnelshift_r(lo, hf, sh);
    const unsigned f24 = __funnelshift_r(lo, hf, sh - 24) & 0xFFFFFFu;
    f = (float)f24 * (1.0f / 16777216.0f);
  } else {
    const int2 s = split_u_slow(u);
    c = s.x;
    f = __int_as_float(s.y);
  }
}

__device__ __forceinline__ bool in_grid_cell(const MixedArgs &A, int cx, int cy) {
  return cx >= 0 && cy >= 0 && cx < A.nx && cy < A.ny;
}

// A point exactly on the grid's far edge (where a plane at the grid bound
// projects it) is taken as the last cell at fraction 1: the same weights and
// no node beyond the grid (the reference's stencil would reach one node past
// its arrays there, with weight 0).
__device__ __forceinline__ void far_edge(int n, int &c, float &f) {
  if (c == n && f == 0.0f) {
    c = n - 1;
    f = 1.0f;
  }
}

// Elastic prediction + Drucker-Prager plastic correction on offset-form
// strain (ConstitutiveModel.cpp:19-81, MaterialPoints.cpp:324-369).
// B = be - I; det(I + B) = 1 + t with t = tr B + det B.
__device__ __forceinline__ void constitutive_update(float4 &s, int &jh, float Lxx,
                                                    float Lxy, float Lyx, float Lyy,
                                                    float dt, float kappa, float mu,
                                                    float alpha) {
  const float J = 1.0f + s.x;
  float bxx = s.x + J * s.y, bxy = J * s.z, byy = s.x + J * s.w;
  // be* = be + dt (L be + be L^T) with be = I + B
  const float LBxx = Lxx * bxx + Lxy * bxy, LBxy = Lxx * bxy + Lxy * byy;
  const float LByx = Lyx * bxx + Lyy * bxy, LByy = Lyx * bxy + Lyy * byy;
  bxx += dt * (2.0f * Lxx + 2.0f * LBxx);
  bxy += dt * ((Lxy + Lyx) + (LBxy + LByx));
  byy += dt * (2.0f * Lyy + 2.0f * LByy);
  float t = (bxx + byy) + (bxx * byy - bxy * bxy);
  float dJ = t / (1.0f + sqrtf(1.0f + t));
  if (jh != 0) {
    if (dJ > 0.0f) { // J > 1: be = J I (ConstitutiveModel.cpp:28-35)
      s = make_float4(dJ, 0.0f, 0.0f, 0.0f);
      return;
    }
    jh = 0;
  }
  const float Js = 1.0f + dJ;
  const float ys = fmaxf(0.0f, -0.5f * alpha * kappa * (2.0f + dJ) * dJ);
  const float htr = 0.5f * (bxx + byy);
  const float dxx = bxx - htr, dyy = byy - htr, dxy = bxy;
  const float dn = sqrtf(dxx * dxx + 2.0f * dxy * dxy + dyy * dyy);
  if (mu * dn > ys * Js) {
    const float l2 = ys * Js / (mu * dn);
    const float detdev = dxx * dyy - dxy * dxy;
    const float l1sq_m1 = t - l2 * l2 * detdev;
    const float l1m1 = l1sq_m1 / (1.0f + sqrtf(1.0f + l1sq_m1));
    bxx = l1m1 + l2 * dxx;
    byy = l1m1 + l2 * dyy;
    bxy = l2 * dxy;
    t = (bxx + byy) + (bxx * byy - bxy * bxy);
    dJ = t / (1.0f + sqrtf(1.0f + t));
  }
  const float inv = 1.0f / (1.0f + dJ);
  s = make_float4(dJ, (bxx - dJ) * inv, bxy * inv, (byy - dJ) * inv);
}

// Kirchhoff stress tau (ConstitutiveModel.cpp:83-97 via
// MaterialPoints.cpp:183-202) scaled to the node force factor -V tau / h.
__device__ __forceinline__ void stress_factor(const float4 s, int jh, float V,
                                              float inv_h, float kappa, float mu,
                                              float &s00, float &s01, float &s11) {
  if (s.x > 0.0f || jh != 0) {
    s00 = s01 = s11 = 0.0f;
    return;
  }
  const float vol = kappa * 0.5f * (2.0f + s.x) * s.x;
  const float dev = 0.5f * (s.y - s.w);
  const float c = -V * inv_h;
  s00 = c * (vol + mu * dev);
  s11 = c * (vol - mu * dev);
  s01 = c * (mu * s.z);
}

struct PRec {
  float4 a; // fx, fy, m, m vx
  float4 b; // m vy, s00, s01, s11
};

__device__ __forceinline__ void scatter_global(const MixedArgs &A, int cx, int cy,
                                               const PRec &r) {
  const int row = A.nx + 1;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int dx = k & 1, dy = k >> 1;
    const int ix = cx + dx, iy = cy + dy;
    const float wx = dx ? r.a.x : 1.0f - r.a.x;
    const float wy = dy ? r.a.y : 1.0f - r.a.y;
    const float w = wx * wy;
    const float gx = dx ? wy : -wy, gy = dy ? wx : -wx;
    float4 add = make_float4(w * r.a.w, w * r.b.x, 0.0f, 0.0f);
    if (w != 0.0f) {
      add.z = r.b.y * gx + r.b.z * gy;
      add.w = r.b.z * gx + r.b.w * gy;
    }
    const int64_t node = (int64_t)iy * row + ix;
    if (!HG_INDEX_OK(node, (int64_t)row * (A.ny + 1), A.status)) continue;
    atomicAdd(&A.accm[node], w * r.a.z);
    atomicAdd(&A.acc4[node], add);
  }
}

// Adds the P2G contribution of one material point at cell (cx, cy) with
// fractions (fx, fy) to 4 corner accumulators a[corner * 5 + {m, px, py, fx, fy}]
// (corner = dx + 2 dy). The internal force is skipped where the weight is
// zero, like PhysicsGrid::computeForces (PhysicsGrid.cpp:439-441).
__device__ __forceinline__ void p2g_corners(const PRec &r, float *a) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int dx = k & 1, dy = k >> 1;
    const float wx = dx ? r.a.x : 1.0f - r.a.x;
    const float wy = dy ? r.a.y : 1.0f - r.a.y;
    const float w = wx * wy;
    a[5 * k + 0] += w * r.a.z;
    a[5 * k + 1] += w * r.a.w;
    a[5 * k + 2] += w * r.b.x;
    // nodes of zero weight get no force (PhysicsGrid.cpp:443-445)
    const bool on = w != 0.0f;
    const float gx = on ? (dx ? wy : -wy) : 0.0f, gy = on ? (dy ? wx : -wx) : 0.0f;
    a[5 * k + 3] += r.b.y * gx + r.b.z * gy;
    a[5 * k + 4] += r.b.z * gx + r.b.w * gy;
  }
}

// Exact float -> double widening with integer operations (keeps the FP64 pipe
// free). Zero and subnormal inputs give 0; they are below the resolution of
// any position they are added to.
__device__ __noinline__ double widen_slow(float f) { return (double)f; }

__device__ __forceinline__ double widen(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if (e == 0u) return 0.0;
  if (e == 0xFFu) return widen_slow(f);
  const unsigned m = b & 0x7FFFFFu;
  const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | (m >> 3);
  return __hiloint2double((int)hi, (int)(m << 29));
}

// Signed distance n . (u - x) of a position in grid units from a plane, each
// product and sum rounded on its own (no contraction into FMA), so that a
// point lying on a plane gives 0 as in the reference's expression
// (MaterialPoints.cpp:381).
__device__ __forceinline__ double plane_distance_u(const MpmPlaneDev &pl, double ux, double uy) {
  return __dadd_rn(__dmul_rn(pl.n[0], __dsub_rn(ux, pl.ux[0])),
                   __dmul_rn(pl.n[1], __dsub_rn(uy, pl.ux[1])));
}

// PhysicsGrid::resolvePlaneCollisions' test of node (ix, iy)
// (PhysicsGrid.cpp:614-629) on the node's world position
// computeGridPointLocation = min + h (i, j) (PhysicsGrid.cpp:71-74), with the
// reference's operations rounded one by one: true when the plane acts on the
// node. Nodes on a plane or on its lower bound decide as in the reference.
__device__ __forceinline__ bool node_behind_plane(const MixedArgs &A, const MpmPlaneDev &pl,
                                                  int ix, int iy) {
  const double px = __dadd_rn(A.gmin[0], __dmul_rn(A.h, (double)ix));
  const double py = __dadd_rn(A.gmin[1], __dmul_rn(A.h, (double)iy));
  if (py < pl.lower_bound) return false;
  const double d = __dadd_rn(__dmul_rn(pl.n[0], __dsub_rn(px, pl.x[0])),
                             __dmul_rn(pl.n[1], __dsub_rn(py, pl.x[1])));
  return !(d > 0.0);
}

__device__ __forceinline__ bool finite_d(double x) {
  return ((unsigned)__double2hiint(x) & 0x7FF00000u) != 0x7FF00000u;
}

// Cell-major fused kernel. A CTA owns one tile of BIN x BIN cells at a time
// and one thread owns one cell: it updates the material points sorted into
// that cell (G2P of this step) and accumulates their P2G contributions for the
// next step in registers, per corner node of the cell. Points that have left
// their cell since the last re-sort go through shared-memory atomics on the
// tile's node window (or global atomics outside it). Corner sums are combined
// per node through shared memory and flushed with one global atomic per node
// and field.
struct FusedSmem {
  float4 va[VA_W * VA_W];
  float slow[5][ACC_W * ACC_W];
  float corner[20][BIN_CELLS];
  unsigned out[2]; // left the tile window / left the sorted cell
};

// One tile of one scene; A lives in shared memory.
template <bool PRIME>
__device__ __forceinline__ void fused_tile(const MixedArgs &A, const int bin, FusedSmem &S) {
  static_assert(THREADS == BIN_CELLS, "one thread per cell of a tile");
  float4 *s_va = S.va;
  float(&s_slow)[5][ACC_W * ACC_W] = S.slow;
  float(&s_corner)[20][BIN_CELLS] = S.corner;
  unsigned *s_out = S.out;
  const int tid = threadIdx.x;
  const int row = A.nx + 1;
  const int lcx = tid % BIN, lcy = tid / BIN;
  {
    const int X0 = (bin % A.ntx) * BIN, Y0 = (bin / A.ntx) * BIN;
    const int WX = X0 - DRIFT - 1, WY = Y0 - DRIFT - 1; // P2G window origin (node)
    if (!PRIME) {
      for (int k = tid; k < VA_W * VA_W; k += THREADS) {
        const int ix = X0 - DRIFT + k % VA_W, iy = Y0 - DRIFT + k / VA_W;
        float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ix >= 0 && iy >= 0 && ix <= A.nx && iy <= A.ny)
          val = A.va[iy * row + ix]; // MIXED grids have < 2^30 nodes
        s_va[k] = val;
      }
    }
    // s_slow is zero here: zeroed at kernel start and by the previous
    // tile's flush
    if (tid < 2) s_out[tid] = 0;
    int ps = A.offsets[bin * BIN_CELLS + tid];
    int pe = A.offsets[bin * BIN_CELLS + tid + 1];
    if (!HG_INDEX_OK(ps, (int64_t)A.n + 1, A.status) || !HG_INDEX_OK(pe, (int64_t)A.n + 1, A.status))
      ps = pe = 0;
    const int gcx = X0 + lcx, gcy = Y0 + lcy;
    // Planes that can touch a point of this tile's window: the window corners
    // bound every position a point of the tile can take this step.
    unsigned plane_mask = 0;
    for (int k = 0; k < A.nplanes; ++k) {
      const MpmPlaneDev &pl = A.planes[k];
      const float x0 = (float)WX, y0 = (float)WY;
      const float x1 = (float)(WX + ACC_W), y1 = (float)(WY + ACC_W);
      float dmin = fminf(fminf(pl.fn[0] * (x0 - pl.fux[0]) + pl.fn[1] * (y0 - pl.fux[1]),
                               pl.fn[0] * (x1 - pl.fux[0]) + pl.fn[1] * (y0 - pl.fux[1])),
                         fminf(pl.fn[0] * (x0 - pl.fux[0]) + pl.fn[1] * (y1 - pl.fux[1]),
                               pl.fn[0] * (x1 - pl.fux[0]) + pl.fn[1] * (y1 - pl.fux[1])));
      if (dmin <= 2.0f * A.pmargin && y1 >= pl.fulb - A.pmargin) plane_mask |= 1u << k;
    }
    // the next point's state is loaded while the current one is processed;
    // the first one before the barrier, under the window loads
    double2 nu = make_double2(0.0, 0.0);
    float2 nmv = make_float2(0.f, 0.f), nvel = make_float2(0.f, 0.f);
    float4 nst = make_float4(0.f, 0.f, 0.f, 0.f);
    int nfl = 0;
    if (ps < pe) {
      nu = A.u[ps];
      nmv = A.mv[ps];
      nvel = A.v[ps];
      nst = A.strain[ps];
      nfl = A.flags[ps];
    }
    __syncthreads();
    float acc[20];
#pragma unroll
    for (int k = 0; k < 20; ++k) acc[k] = 0.f;
    // per-thread counters and flags, published once after the loop
    unsigned left_window = 0, left_cell = 0;
    bool nonfinite = false;
    for (int p = ps; p < pe; ++p) {
      const double2 u = nu;
      const float2 mv = nmv;
      float2 vel = nvel;
      float4 st = nst;
      const int fl = nfl;
      if (p + 1 < pe) { // (an unconditional reload of the last point was slower)
        nu = A.u[p + 1];
        nmv = A.mv[p + 1];
        nvel = A.v[p + 1];
        nst = A.strain[p + 1];
        nfl = A.flags[p + 1];
      }
      int cx, cy;
      float fx, fy;
      split_u(u.x, cx, fx);
      split_u(u.y, cy, fy);
      if (!in_grid_cell(A, cx, cy)) { // the grid's far edge, or outside it
        far_edge(A.nx, cx, fx);
        far_edge(A.ny, cy, fy);
        if (!in_grid_cell(A, cx, cy)) {
          atomicOr(A.status, (uint32_t)HG_STATUS_OUT_OF_GRID);
          continue;
        }
      }
      int jh = fl & 1;
      int ncx = cx, ncy = cy;
      float nfx = fx, nfy = fy;
      if (!PRIME) {
        float4 n00, n10, n01, n11;
        const int gx = cx - (X0 - DRIFT), gy = cy - (Y0 - DRIFT);
        const bool in_window = gx >= 0 && gy >= 0 && gx <= VA_W - 2 && gy <= VA_W - 2;
        if (in_window) {
          const int k0 = gy * VA_W + gx;
          n00 = s_va[k0];
          n10 = s_va[k0 + 1];
          n01 = s_va[k0 + VA_W];
          n11 = s_va[k0 + VA_W + 1];
        } else {
          const int k0 = cy * row + cx;
          if (HG_INDEX_OK(k0 + row + 1, (int64_t)row * (A.ny + 1), A.status)) {
            n00 = A.va[k0];
            n10 = A.va[k0 + 1];
            n01 = A.va[k0 + row];
            n11 = A.va[k0 + row + 1];
          } else {
            n00 = n10 = n01 = n11 = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
        const float wx0 = 1.0f - fx, wx1 = fx, wy0 = 1.0f - fy, wy1 = fy;
        const float w00 = wx0 * wy0, w10 = wx1 * wy0, w01 = wx0 * wy1, w11 = wx1 * wy1;
        // velocity gradient from the grid-unit weight gradients
        const float ih = A.inv_h;
        const float Lxx = (-wy0 * n00.x + wy0 * n10.x - wy1 * n01.x + wy1 * n11.x) * ih;
        const float Lxy = (-wx0 * n00.x - wx1 * n10.x + wx0 * n01.x + wx1 * n11.x) * ih;
        const float Lyx = (-wy0 * n00.y + wy0 * n10.y - wy1 * n01.y + wy1 * n11.y) * ih;
        const float Lyy = (-wx0 * n00.y - wx1 * n10.y + wx0 * n01.y + wx1 * n11.y) * ih;
        const float vpx = w00 * n00.x + w10 * n10.x + w01 * n01.x + w11 * n11.x;
        const float vpy = w00 * n00.y + w10 * n10.y + w01 * n01.y + w11 * n11.y;
        const float apx = w00 * n00.z + w10 * n10.z + w01 * n01.z + w11 * n11.z;
        const float apy = w00 * n00.w + w10 * n10.w + w01 * n01.w + w11 * n11.w;
        constitutive_update(st, jh, Lxx, Lxy, Lyx, Lyy, A.dt, A.kappa, A.mu, A.dp_alpha);
        // kinematically scripted points move with their own velocity
        const bool kin = (fl & 2) != 0;
        const float dtih = A.dt * A.inv_h;
        const float dux = dtih * (kin ? vel.x : vpx);
        const float duy = dtih * (kin ? vel.y : vpy);
        {
          const float a = A.flip_alpha;
          const float fvx = (1.0f - a) * vpx + a * (vel.x + A.dt * apx);
          const float fvy = (1.0f - a) * vpy + a * (vel.y + A.dt * apy);
          vel.x = kin ? vel.x : fvx;
          vel.y = kin ? vel.y : fvy;
        }
        double2 un = make_double2(u.x + widen(dux), u.y + widen(duy));
        // new cell and fraction by FP32 carry of the old fraction
        nfx = fx + dux;
        nfy = fy + duy;
        bool exact = !(fabsf(dux) < 1.0f && fabsf(duy) < 1.0f);
        // the tile's plane mask bounds points that start in the window and
        // move less than a cell; any other point tests every plane
        const unsigned pmask = (in_window && !exact) ? plane_mask : (1u << A.nplanes) - 1u;
        {
          const float cx1 = floorf(nfx), cy1 = floorf(nfy); // -1, 0 or 1
          ncx += (int)cx1;
          ncy += (int)cy1;
          nfx -= cx1;
          nfy -= cy1;
        }
        // MaterialPoints::resolvePlaneCollisions in grid units; FP32 test
        // first, FP64 where the point is within pmargin cells of a plane
        const float ufx = (float)ncx + nfx, ufy = (float)ncy + nfy;
        for (unsigned mk = pmask; mk; mk &= mk - 1) {
          const MpmPlaneDev &pl = A.planes[__ffs(mk) - 1];
          if (ufy < pl.fulb - A.pmargin) continue;
          const float dapprox = pl.fn[0] * (ufx - pl.fux[0]) + pl.fn[1] * (ufy - pl.fux[1]);
          if (dapprox > A.pmargin) continue;
          if (un.y < pl.ulb) continue;
          const double d = plane_distance_u(pl, un.x, un.y);
          if (d > 0.0) continue;
          un.x += -d * pl.n[0];
          un.y += -d * pl.n[1];
          exact = true;
          if (!pl.sticking) {
            const float vn = pl.fn[0] * vel.x + pl.fn[1] * vel.y;
            if (vn > 0.0f) continue;
            vel.x -= vn * pl.fn[0];
            vel.y -= vn * pl.fn[1];
          } else {
            vel = make_float2(0.0f, 0.0f);
          }
        }
        if (exact || !in_grid_cell(A, ncx, ncy)) {
          // (also when the FP32 carry put a point just inside the low edge in
          // cell -1, its fraction rounded down and its step rounded up: the
          // FP64 position decides)
          split_u(un.x, ncx, nfx);
          split_u(un.y, ncy, nfy);
          far_edge(A.nx, ncx, nfx);
          far_edge(A.ny, ncy, nfy);
        }
        // the position stays finite while its increments do (it was finite
        // and inside the grid): one test covers position, velocity and J
        nonfinite |= !isfinite((dux + duy) + (vel.x + vel.y) + st.x);
        A.u[p] = un;
        A.v[p] = vel;
        A.strain[p] = st;
        A.flags[p] = (uint8_t)((fl & ~1) | jh);
        if ((ncx != gcx) | (ncy != gcy)) { // a point in its sorted cell is in the window
          const int ngx = ncx - (X0 - DRIFT), ngy = ncy - (Y0 - DRIFT);
          left_window += (ngx < 0) | (ngy < 0) | (ngx > VA_W - 2) | (ngy > VA_W - 2);
          ++left_cell;
        }
      }
      if (!in_grid_cell(A, ncx, ncy)) {
        atomicOr(A.status, (uint32_t)HG_STATUS_OUT_OF_GRID);
        continue;
      }
      // ---- P2G contribution for the next step ----
      PRec r;
      float s00, s01, s11;
      stress_factor(st, jh, mv.y, A.inv_h, A.kappa, A.mu, s00, s01, s11);
      r.a = make_float4(nfx, nfy, mv.x, mv.x * vel.x);
      r.b = make_float4(mv.x * vel.y, s00, s01, s11);
      if (ncx == gcx && ncy == gcy) {
        p2g_corners(r, acc);
      } else {
        const int lx = ncx - WX, ly = ncy - WY;
        if (lx >= 0 && ly >= 0 && lx <= ACC_W - 2 && ly <= ACC_W - 2) {
          float part[20];
#pragma unroll
          for (int k = 0; k < 20; ++k) part[k] = 0.f;
          p2g_corners(r, part);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int node = (ly + (k >> 1)) * ACC_W + lx + (k & 1);
#pragma unroll
            for (int c = 0; c < 5; ++c) atomicAdd(&s_slow[c][node], part[5 * k + c]);
          }
        } else {
          scatter_global(A, ncx, ncy, r);
        }
      }
    }
    if (nonfinite) atomicOr(A.status, (uint32_t)HG_STATUS_NONFINITE);
    if (left_window) atomicAdd(&s_out[0], left_window);
    if (left_cell) atomicAdd(&s_out[1], left_cell);
#pragma unroll
    for (int k = 0; k < 20; ++k) s_corner[k][tid] = acc[k];
    __syncthreads();
    // ---- node sums of the tile window, flushed to the global accumulators ----
    for (int k = tid; k < ACC_W * ACC_W; k += THREADS) {
      const int i = k % ACC_W, j = k / ACC_W;
      float sum[5];
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        sum[c] = s_slow[c][k];
        s_slow[c][k] = 0.f; // ready for the next tile
      }
      const int bi = i - (DRIFT + 1), bj = j - (DRIFT + 1); // node index within the tile
      if (bi >= 0 && bj >= 0 && bi <= BIN && bj <= BIN) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int dx = q & 1, dy = q >> 1;
          const int ci = bi - dx, cj = bj - dy;
          if (ci < 0 || cj < 0 || ci >= BIN || cj >= BIN) continue;
          const int cell = cj * BIN + ci;
#pragma unroll
          for (int c = 0; c < 5; ++c) sum[c] += s_corner[5 * q + c][cell];
        }
      }
      if (sum[0] == 0.f && sum[1] == 0.f && sum[2] == 0.f && sum[3] == 0.f && sum[4] == 0.f)
        continue;
      const int ix = WX + i, iy = WY + j;
      if (ix < 0 || iy < 0 || ix > A.nx || iy > A.ny) continue;
      const int node = iy * row + ix;
      if (!HG_INDEX_OK(node, (int64_t)row * (A.ny + 1), A.status)) continue;
      atomicAdd(&A.accm[node], sum[0]);
      atomicAdd(&A.acc4[node], make_float4(sum[1], sum[2], sum[3], sum[4]));
    }
    __syncthreads();
    if (tid < 2 && s_out[tid]) atomicAdd(&A.outside[tid], s_out[tid]);
  }
}

// fused_tile expects the moved-point window to be zero on entry (it leaves
// it zero); the first tile's barrier orders this against its use.
__device__ __forceinline__ void zero_slow(FusedSmem &S) {
  float *s = &S.slow[0][0];
  for (int k = threadIdx.x; k < 5 * ACC_W * ACC_W; k += THREADS) s[k] = 0.f;
}

template <bool PRIME>
__global__ void __launch_bounds__(THREADS, 3) kx_g2p2g(const __grid_constant__ MixedArgs A) {
  // the arguments stay in the constant bank: operands need no registers
  __shared__ FusedSmem S;
  zero_slow(S);
  // launched with programmatic dependence on the grid update before it: only
  // shared memory is touched before the wait
  pdl_wait();
  pdl_trigger();
  const int nact = *A.nactive;
  for (int t = blockIdx.x; t < nact; t += gridDim.x) {
    const int tile = A.active[t];
    if (!HG_INDEX_OK(tile, (int64_t)A.ntx * A.nty, A.status)) continue;
    fused_tile<PRIME>(A, tile, S);
  }
}

// Exclusive prefix of the scenes' work-item counts, in shared memory
// (nslots <= MAX_BATCH). Item k of the launch is tile (k - prefix[s]) of
// scene s with prefix[s] <= k < prefix[s + 1].
__device__ __forceinline__ void batch_prefix(const MixedArgs *slots, int nslots, int *prefix) {
  __shared__ int warp_tot[THREADS / 32];
  constexpr int PER = (MAX_BATCH + THREADS - 1) / THREADS;
  int v[PER];
  int sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int s = threadIdx.x * PER + j;
    v[j] = s < nslots ? *slots[s].nactive : 0;
    sum += v[j];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  int off = 0;
  for (int w = 0; w < wid; ++w) off += warp_tot[w];
  int run = off + x - sum;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    prefix[threadIdx.x * PER + j] = run;
    run += v[j];
  }
  if (threadIdx.x == THREADS - 1) prefix[THREADS * PER] = run;
  __syncthreads();
}

constexpr int PREFIX_LEN = ((MAX_BATCH + THREADS - 1) / THREADS) * THREADS + 1;

// Copies slot s's arguments into shared memory with all threads, up to the
// planes in use (the arguments end with the plane array).
__device__ __forceinline__ void load_slot(const MixedArgs *slots, int s, MixedArgs &A) {
  __syncthreads(); // the previous tile is done with A
  const int words = (int)((offsetof(MixedArgs, planes) +
                           (size_t)slots[s].nplanes * sizeof(MpmPlaneDev) + 15) / 16);
  const int4 *src = reinterpret_cast<const int4 *>(slots + s);
  int4 *dst = reinterpret_cast<int4 *>(&A);
  for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
  __syncthreads();
}

__device__ __forceinline__ int batch_slot(const int *prefix, int nslots, int item) {
  int lo = 0, hi = nslots - 1;
  while (lo < hi) { // largest s with prefix[s] <= item
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Work queue of a batched launch over its (scene, tile) items. q[0] is the
// next unclaimed item and q[1] counts the CTAs that found the queue empty;
// the last of those resets both, so every launch (ordered after the previous
// one on the stream) starts from zero. Thread 0 claims guided chunks: about
// a 1/(2 x CTAs) share of what it last saw remaining, 1 to QUEUE_MAX_CHUNK
// items, so that early claims keep consecutive items (one scene's tiles)
// together and the last ones balance the tail one tile at a time. Tiles
// differ widely in point count across scenes of 2e3 to 2e5 points, which a
// static split by item count cannot balance.
constexpr int QUEUE_MAX_CHUNK = 8;

__device__ __forceinline__ int2 queue_claim(int32_t *q, int total, int seen) {
  const int g = max(1, min(QUEUE_MAX_CHUNK, (total - seen) / (2 * (int)gridDim.x)));
  return make_int2(atomicAdd(q, g), g);
}

__device__ __forceinline__ void queue_done(int32_t *q) {
  if (threadIdx.x != 0) return;
  __threadfence();
  if (atomicAdd(q + 1, 1) == (int)gridDim.x - 1) {
    q[0] = 0;
    q[1] = 0;
  }
}

// Drains the queue: tile(A, tile index) for every claimed item, the scene's
// arguments copied into A whenever the item's scene changes. The next chunk
// is claimed while this one runs.
template <class F>
__device__ __forceinline__ void drain_queue(const MixedArgs *slots, int nslots, const int *prefix,
                                            int32_t *q, MixedArgs &A, F &&tile) {
  __shared__ int2 s_claim;
  const int total = prefix[nslots];
  int2 claim = threadIdx.x == 0 ? queue_claim(q, total, 0) : make_int2(0, 0);
  int s = -1;
  for (;;) {
    if (threadIdx.x == 0) s_claim = claim;
    __syncthreads();
    const int2 c = s_claim;
    __syncthreads();
    if (c.x >= total) break;
    if (threadIdx.x == 0) claim = queue_claim(q, total, c.x + c.y);
    const int end = min(c.x + c.y, total);
    for (int item = c.x; item < end; ++item) {
      if (s < 0 || item >= prefix[s + 1] || item < prefix[s]) {
        s = batch_slot(prefix, nslots, item);
        load_slot(slots, s, A);
      }
      tile(A, A.active[item - prefix[s]]);
    }
  }
  queue_done(q);
}


// All scenes of a batch in one launch: the CTAs drain (scene, tile) items.
__global__ void __launch_bounds__(THREADS, 3) kb_g2p2g(const MixedArgs *__restrict__ slots,
                                                     int nslots, int32_t *queue) {
  __shared__ FusedSmem S;
  __shared__ MixedArgs A;
  __shared__ int prefix[PREFIX_LEN];
  zero_slow(S);
  batch_prefix(slots, nslots, prefix);
  drain_queue(slots, nslots, prefix, queue, A,
              [&](const MixedArgs &a, int tile) { fused_tile<false>(a, tile, S); });
}

// ---- MIXED step with the uGIMP basis --------------------------------------
//
// uGIMPLinearBasisFunctions (uGIMPLinearBasisFunctions.cpp:6-156) in FP32
// grid units: the weight of node i along one axis is the hat function
// integrated over the point's extent [u - hl, u + hl], divided by 2 hl, with
// derivative d/du; for hl <= 1/2 a point of fraction f in cell c touches the
// nodes c-1 (f < hl), c, c+1 and c+2 (f > 1 - hl). The kernel below shares
// the linear path's sorting, active tiles, grid update and chunk graphs.

// Weights and derivatives along one axis of the three nodes b .. b+2 that
// can carry weight when hl <= 1/2: b = c - 1 for f < 1/2 (node c+2 then has
// none, |f - 2| >= 1 + hl) and b = c otherwise (node c-1 has none). Each
// node's offset is f - k as in the reference's stencil over c-1 .. c+2.
// False if a node of non-zero weight lies outside 0 .. n (the reference's
// stencil would leave its grid).
__device__ __forceinline__ bool ugimp_axis(int c, float f, float hl, int n, int &b, float w[3],
                                           float g[3]) {
  const int up = f >= 0.5f ? 1 : 0;
  b = c - 1 + up;
  // With a = |d|, d = u - x_i, and i2 = 1 / (2 hl) (lin_integral and
  // lin_integral_grad with unit weight): w = 0 for a >= 1 + hl;
  // w = (1 + hl - a)^2 i2 / 2, dw/du = -sign(d) (1 + hl - a) i2 for
  // a >= 1 - hl; w = 2 hl (1 - a) i2, dw/du = -sign(d) 2 hl i2 for a >= hl;
  // else w = (2 hl - (hl^2 + a^2)) i2, dw/du = -2 d i2. The middle node lies
  // within 1/2 of the point and the outer two at least 1/2 away (>= hl), so
  // each takes only the cases it can reach. The cases are selected, not
  // branched on (the lanes of a warp take different ones).
  const float i2 = 0.5f / hl, h2 = 2.0f * hl, h2i2 = h2 * i2;
#pragma unroll
  for (int m = 0; m < 3; m += 2) {
    const float d = f - (float)(m - 1 + up);
    const float a = fabsf(d), sg = d >= 0.0f ? 1.0f : -1.0f;
    const float t = 1.0f + hl - a;
    const bool out = a >= 1.0f + hl, edge = a >= 1.0f - hl;
    w[m] = out ? 0.0f : (edge ? 0.5f * t * t * i2 : (1.0f - a) * h2i2);
    g[m] = out ? 0.0f : (edge ? -sg * t * i2 : -sg * h2i2);
  }
  {
    const float d = f - (float)up;
    const float a = fabsf(d), sg = d >= 0.0f ? 1.0f : -1.0f;
    // (at a = 1 - hl = hl = 1/2 the two cases agree)
    const bool far = a >= hl;
    w[1] = far ? (1.0f - a) * h2i2 : (h2 - (hl * hl + a * a)) * i2;
    g[1] = far ? -sg * h2i2 : -2.0f * d * i2;
  }
  if (c >= 1 && c + 2 <= n) return true; // nodes c-1 .. c+2 all on the grid
  bool ok = true;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int i = b + m;
    if ((w[m] != 0.0f || g[m] != 0.0f) && (i < 0 || i > n)) ok = false;
  }
  return ok;
}

// Nodes of a 3-node axis that carry weight or derivative (a node is in the
// point's support when it does along both axes; outside it, it may lie off
// the grid)
__device__ __forceinline__ unsigned ugimp_support(const float w[3], const float g[3]) {
  return (w[0] != 0.0f || g[0] != 0.0f ? 1u : 0u) | (w[1] != 0.0f || g[1] != 0.0f ? 2u : 0u) |
         (w[2] != 0.0f || g[2] != 0.0f ? 4u : 0u);
}

// One thread per point, in the sorted order: a warp's points lie in a few
// neighbouring cells, so its gathers from the grid and its P2G atomics (one
// float4 and one float reduction per node) stay within a few cache lines.
// Each point has its own half-width (ResamplingTools.cpp:58-104 assigns them
// to inserted points). Planes take the linear kernel's FP32 test first and
// the FP64 test only within pmargin cells of a plane. (A tile-window form of
// this kernel, with shared-memory G2P and P2G, was slower: five shared
// atomics per node against two global reductions, at a third of the
// occupancy.)
template <bool PRIME>
__global__ void __launch_bounds__(THREADS) kxu_step(const __grid_constant__ MixedArgs A) {
  // launched with programmatic dependence on the grid update before it
  pdl_wait();
  pdl_trigger();
  const int row = A.nx + 1;
  [[maybe_unused]] const int64_t nn = (int64_t)row * (A.ny + 1); // bounds-checked builds
  unsigned moved = 0;
  bool nonfinite = false;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.n;
       p += (int64_t)gridDim.x * blockDim.x) {
    double2 un = A.u[p];
    const float2 mv = A.mv[p];
    float2 vel = A.v[p];
    float4 st = A.strain[p];
    const int fl = A.flags[p];
    const float hl = A.hl[p];
    int jh = fl & 1;
    int cx, cy;
    float fx, fy;
    split_u(un.x, cx, fx);
    split_u(un.y, cy, fy);
    far_edge(A.nx, cx, fx);
    far_edge(A.ny, cy, fy);
    int bx, by;
    float wx[3], gx[3], wy[3], gy[3];
    if (!in_grid_cell(A, cx, cy) || !ugimp_axis(cx, fx, hl, A.nx, bx, wx, gx) ||
        !ugimp_axis(cy, fy, hl, A.ny, by, wy, gy)) {
      atomicOr(A.status, (uint32_t)HG_STATUS_OUT_OF_GRID);
      continue;
    }
    if (!PRIME) {
      // ---- G2P of this step at the start-of-step position ----
      float Lxx = 0.f, Lxy = 0.f, Lyx = 0.f, Lyy = 0.f, vpx = 0.f, vpy = 0.f, apx = 0.f,
            apy = 0.f;
      const unsigned sx = ugimp_support(wx, gx), sy = ugimp_support(wy, gy);
#pragma unroll
      for (int ky = 0; ky < 3; ++ky) {
#pragma unroll
        for (int kx = 0; kx < 3; ++kx) {
          if (!((sx >> kx) & (sy >> ky) & 1u)) continue; // outside the support
          const float w = wx[kx] * wy[ky], dX = gx[kx] * wy[ky], dY = wx[kx] * gy[ky];
          const int node = (by + ky) * row + (bx + kx); // MIXED grids have < 2^30 nodes
          if (!HG_INDEX_OK(node, nn, A.status)) continue;
          const float4 nv = A.va[node];
          Lxx += nv.x * dX;
          Lxy += nv.x * dY;
          Lyx += nv.y * dX;
          Lyy += nv.y * dY;
          vpx += w * nv.x;
          vpy += w * nv.y;
          apx += w * nv.z;
          apy += w * nv.w;
        }
      }
      const float ih = A.inv_h;
      constitutive_update(st, jh, Lxx * ih, Lxy * ih, Lyx * ih, Lyy * ih, A.dt, A.kappa, A.mu,
                          A.dp_alpha);
      const bool kin = (fl & 2) != 0;
      const float dtih = A.dt * A.inv_h;
      const float dux = dtih * (kin ? vel.x : vpx);
      const float duy = dtih * (kin ? vel.y : vpy);
      {
        const float a = A.flip_alpha;
        const float fvx = (1.0f - a) * vpx + a * (vel.x + A.dt * apx);
        const float fvy = (1.0f - a) * vpy + a * (vel.y + A.dt * apy);
        vel.x = kin ? vel.x : fvx;
        vel.y = kin ? vel.y : fvy;
      }
      un = make_double2(un.x + widen(dux), un.y + widen(duy));
      // new cell and fraction by FP32 carry of the old fraction, as in the
      // linear kernel; the FP64 position decides after a plane projection,
      // a move of a cell or more, or a carry that leaves the grid
      bool exact = !(fabsf(dux) < 1.0f && fabsf(duy) < 1.0f);
      int ncx = cx, ncy = cy;
      float nfx = fx + dux, nfy = fy + duy;
      {
        const float cx1 = floorf(nfx), cy1 = floorf(nfy); // -1, 0 or 1
        ncx += (int)cx1;
        ncy += (int)cy1;
        nfx -= cx1;
        nfy -= cy1;
      }
      // MaterialPoints::resolvePlaneCollisions (MaterialPoints.cpp:371-423) in
      // grid units: FP32 test first, FP64 on the positions within pmargin
      // cells of a plane
      const float ufx = ((float)cx + fx) + dux, ufy = ((float)cy + fy) + duy;
      for (int k = 0; k < A.nplanes; ++k) {
        const MpmPlaneDev &pl = A.planes[k];
        if (ufy < pl.fulb - A.pmargin) continue;
        const float dapprox = pl.fn[0] * (ufx - pl.fux[0]) + pl.fn[1] * (ufy - pl.fux[1]);
        if (dapprox > A.pmargin) continue;
        if (un.y < pl.ulb) continue;
        const double d = plane_distance_u(pl, un.x, un.y);
        if (d > 0.0) continue;
        un.x += -d * pl.n[0];
        un.y += -d * pl.n[1];
        exact = true;
        if (!pl.sticking) {
          const float vn = pl.fn[0] * vel.x + pl.fn[1] * vel.y;
          if (vn > 0.0f) continue;
          vel.x -= vn * pl.fn[0];
          vel.y -= vn * pl.fn[1];
        } else {
          vel = make_float2(0.0f, 0.0f);
        }
      }
      if (exact || !in_grid_cell(A, ncx, ncy)) {
        split_u(un.x, ncx, nfx);
        split_u(un.y, ncy, nfy);
        far_edge(A.nx, ncx, nfx);
        far_edge(A.ny, ncy, nfy);
      }
      // the position stays finite while its increments do (it was finite
      // and inside the grid)
      nonfinite |= !isfinite((dux + duy) + (vel.x + vel.y) + st.x);
      A.u[p] = un;
      A.v[p] = vel;
      A.strain[p] = st;
      A.flags[p] = (uint8_t)((fl & ~1) | jh);
      moved += (ncx != cx) | (ncy != cy);
      if (!in_grid_cell(A, ncx, ncy) || !ugimp_axis(ncx, nfx, hl, A.nx, bx, wx, gx) ||
          !ugimp_axis(ncy, nfy, hl, A.ny, by, wy, gy)) {
        atomicOr(A.status, (uint32_t)HG_STATUS_OUT_OF_GRID);
        continue;
      }
    }
    // ---- P2G contribution for the next step ----
    float s00, s01, s11;
    stress_factor(st, jh, mv.y, A.inv_h, A.kappa, A.mu, s00, s01, s11);
    const float mvx = mv.x * vel.x, mvy = mv.x * vel.y;
    const unsigned sx = ugimp_support(wx, gx), sy = ugimp_support(wy, gy);
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        if (!((sx >> kx) & (sy >> ky) & 1u)) continue; // outside the support
        const float w = wx[kx] * wy[ky];
        const float dX = gx[kx] * wy[ky], dY = wx[kx] * gy[ky];
        const int node = (by + ky) * row + (bx + kx); // MIXED grids have < 2^30 nodes
        if (!HG_INDEX_OK(node, nn, A.status)) continue;
        float4 add = make_float4(w * mvx, w * mvy, 0.0f, 0.0f);
        if (w != 0.0f) { // nodes of zero weight get no force (PhysicsGrid.cpp:439-441)
          add.z = s00 * dX + s01 * dY;
          add.w = s01 * dX + s11 * dY;
        }
        atomicAdd(&A.accm[node], w * mv.x);
        atomicAdd(&A.acc4[node], add);
      }
    }
  }
  if (nonfinite) atomicOr(A.status, (uint32_t)HG_STATUS_NONFINITE);
  // points that changed cell: the re-sort trigger of the linear kernel
  for (int o = 16; o > 0; o >>= 1) moved += __shfl_down_sync(0xffffffffu, moved, o);
  if ((threadIdx.x & 31) == 0 && moved) atomicAdd(&A.outside[1], moved);
}

// Node update of one tile; one thread per node of the 16x16 tile.
__device__ __forceinline__ void update_tile(const MixedArgs &A, const int tile) {
  float4 *va = A.va_out;
  const int row = A.nx + 1;
  const int lx = threadIdx.x % BIN, ly = threadIdx.x / BIN;
  {
    const int ix = (tile % A.ntx) * BIN + lx, iy = (tile / A.ntx) * BIN + ly;
    if (ix > A.nx || iy > A.ny) return;
    const int i = iy * row + ix;
    const float m = A.accm[i];
    const float4 acc = A.acc4[i];
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (m > 0.0f) {
      const float fx = acc.z + m * A.gx, fy = acc.w + m * A.gy;
      // p_new - p, kept as an increment so FP32 keeps its bits on it
      float dpx = A.dt * fx, dpy = A.dt * fy;
      for (int k = 0; k < A.nplanes; ++k) {
        const MpmPlaneDev &pl = A.planes[k];
        const float fy_node = (float)iy;
        if (fy_node < pl.fulb - A.pmargin) continue;
        float d = pl.fn[0] * ((float)ix - pl.fux[0]) + pl.fn[1] * (fy_node - pl.fux[1]);
        if (fabsf(d) < A.pmargin || fabsf(fy_node - pl.fulb) < A.pmargin) {
          // near the plane or its lower bound the reference's own test decides
          if (!node_behind_plane(A, pl, ix, iy)) continue;
          d = -1.0f;
        }
        if (d > 0.0f) continue;
        if (!pl.sticking) {
          const float vx = (acc.x + dpx) / m, vy = (acc.y + dpy) / m;
          const float vn = pl.fn[0] * vx + pl.fn[1] * vy;
          if (vn > 0.0f) continue;
          dpx -= m * vn * pl.fn[0];
          dpy -= m * vn * pl.fn[1];
        } else {
          dpx = -acc.x;
          dpy = -acc.y;
        }
      }
      const float inv_m = 1.0f / m;
      out = make_float4((acc.x + dpx) * inv_m, (acc.y + dpy) * inv_m,
                        dpx * inv_m / A.dt, dpy * inv_m / A.dt);
    }
    va[i] = out;
    A.gm[i] = m;
    A.accm[i] = 0.f;
    A.acc4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

__global__ void __launch_bounds__(THREADS) kx_grid_update(const __grid_constant__ MixedArgs A) {
  // launched with programmatic dependence on the fused kernel before it
  pdl_wait();
  pdl_trigger();
  const int nact = *A.nactive;
  for (int t = blockIdx.x; t < nact; t += gridDim.x) {
    const int tile = A.active[t];
    if (!HG_INDEX_OK(tile, (int64_t)A.ntx * A.nty, A.status)) continue;
    update_tile(A, tile);
  }
}

__global__ void __launch_bounds__(THREADS) kb_grid_update(const MixedArgs *__restrict__ slots,
                                                          int nslots, int32_t *queue) {
  __shared__ MixedArgs A;
  __shared__ int prefix[PREFIX_LEN];
  batch_prefix(slots, nslots, prefix);
  drain_queue(slots, nslots, prefix, queue, A,
              [&](const MixedArgs &a, int tile) { update_tile(a, tile); });
}

// Copies every member's out-of-window counters into one array, for a single
// asynchronous read-back per batch step.
__global__ void kb_gather_outside(const MixedArgs *__restrict__ slots, int nslots,
                                  uint32_t *out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  out[2 * s] = slots[s].outside[0];
  out[2 * s + 1] = slots[s].outside[1];
}

// ---- re-sort -----------------------------------------------------------------

__global__ void kx_keys(int64_t n, int nx, int ny, int ntx, const double2 *__restrict__ u,
                        int32_t *keys, int32_t *counts, uint32_t *status) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  // Cell key floor((x - min)/h) in the reference's form (LinearBasisFunctions.
  // cpp:53-59) is floor(u) here: u was computed with exactly that division.
  const double2 up = u[p];
  int cx = (int)floor(up.x), cy = (int)floor(up.y);
  // a point exactly on the far edge belongs to the last cell
  if (up.x == (double)nx) cx = nx - 1;
  if (up.y == (double)ny) cy = ny - 1;
  if (!(up.x >= 0.0 && up.y >= 0.0 && cx < nx && cy < ny)) {
    atomicOr(status, (uint32_t)HG_STATUS_OUT_OF_GRID);
    cx = min(max(cx, 0), nx - 1);
    cy = min(max(cy, 0), ny - 1);
  }
  const int key = ((cy / BIN) * ntx + cx / BIN) * BIN_CELLS + (cy % BIN) * BIN + (cx % BIN);
  keys[p] = key;
  atomicAdd(&counts[key], 1);
}

__global__ void kx_scatter(int64_t n, const int32_t *__restrict__ keys,
                           const int32_t *__restrict__ offsets, int32_t *cursor,
                           MixedParticles src, MixedParticles dst, int32_t *inv, int32_t *skey) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int key = keys[p];
  const int64_t d = offsets[key] + atomicAdd(&cursor[key], 1);
  const int32_t id = src.id[p];
  dst.u[d] = src.u[p];
  dst.v[d] = src.v[p];
  dst.mv[d] = src.mv[p];
  dst.strain[d] = src.strain[p];
  dst.flags[d] = src.flags[p];
  dst.id[d] = id;
  if (src.hl) dst.hl[d] = src.hl[p];
  // the order tables: ids are upload indices 0 .. n-1
  skey[d] = key;
  if (id >= 0 && id < n) inv[id] = (int32_t)d;
}

__global__ void kx_active(int ntx, int nty, const int32_t *__restrict__ offsets,
                          int32_t *bins, int32_t *tiles, int32_t *nactive) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= ntx * nty) return;
  auto count = [&](int t) {
    return offsets[(t + 1) * BIN_CELLS] - offsets[t * BIN_CELLS];
  };
  if (count(b) > 0) bins[atomicAdd(&nactive[0], 1)] = b;
  const int tx = b % ntx, ty = b / ntx;
  bool any = false;
  for (int dy = -1; dy <= 1 && !any; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      const int x = tx + dx, y = ty + dy;
      if (x < 0 || y < 0 || x >= ntx || y >= nty) continue;
      if (count(y * ntx + x) > 0) {
        any = true;
        break;
      }
    }
  if (any) tiles[atomicAdd(&nactive[1], 1)] = b;
}

// True when tile b is in the active tile set: within one tile of a tile that
// holds points (the tiles the grid update covers).
__device__ __forceinline__ bool tile_active(const int32_t *__restrict__ off, int ntx, int nty,
                                            int b) {
  const int tx = b % ntx, ty = b / ntx;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      const int x = tx + dx, y = ty + dy;
      if (x < 0 || y < 0 || x >= ntx || y >= nty) continue;
      const int t = y * ntx + x;
      if (off[(t + 1) * BIN_CELLS] > off[t * BIN_CELLS]) return true;
    }
  return false;
}

// The grid update writes (va, gm) only on active tiles. After a re-sort,
// nodes of tiles outside the new set are cleared (those still holding a
// mass), so that a tile that dropped out does not keep its last update.
// One block of 256 threads per tile, one thread per node.
__device__ __forceinline__ void clear_inactive_tile(int nx, int ny, int ntx, int nty,
                                                    const int32_t *__restrict__ off, int b,
                                                    float4 *va, float *gm) {
  if (tile_active(off, ntx, nty, b)) return;
  const int ix = (b % ntx) * BIN + (int)threadIdx.x % BIN;
  const int iy = (b / ntx) * BIN + (int)threadIdx.x / BIN;
  if (ix > nx || iy > ny) return;
  const int64_t i = (int64_t)iy * (nx + 1) + ix;
  if (gm[i] != 0.f) {
    gm[i] = 0.f;
    va[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

__global__ void __launch_bounds__(BIN_CELLS) kx_clear_inactive(int nx, int ny, int ntx, int nty,
                                                               const int32_t *__restrict__ off,
                                                               float4 *va, float *gm) {
  for (int b = blockIdx.x; b < ntx * nty; b += gridDim.x)
    clear_inactive_tile(nx, ny, ntx, nty, off, b, va, gm);
}

// ---- batched re-sort -------------------------------------------------------------
//
// The re-sort of every batch member that needs one in a step, in eight launches
// whatever their number: the same counting sort as above, over (member, item)
// work items. The host lays out, per member, the item counts of each pass as
// prefix sums (points, keys, scan chunks, bins); a thread finds its member by
// binary search over them.

struct RebinArgs {
  int64_t n;
  int nx, ny, ntx, nty;
  MixedParticles src, dst;
  int32_t *keys, *counts, *offsets, *cursor, *bins, *tiles, *nactive, *chunk_sums;
  uint32_t *status, *outside;
  float4 *va; // the grid update's outputs (cleared on tiles that leave the set)
  float *gm;
};

struct RebinPrefix {
  const int64_t *pts, *keys, *chunks, *bins; // nmem + 1 each
  int nmem;
};

constexpr int RB_CHUNK = 2048; // elements per scan chunk (256 threads x 8)

__device__ __forceinline__ int member_of(const int64_t *pre, int nmem, int64_t item) {
  int lo = 0, hi = nmem - 1;
  while (lo < hi) { // largest m with pre[m] <= item
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void kr_clear(const RebinArgs *__restrict__ R, RebinPrefix P) {
  const int64_t total = P.keys[P.nmem];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = member_of(P.keys, P.nmem, i);
    const int64_t j = i - P.keys[m]; // 0 .. nkeys
    const RebinArgs &a = R[m];
    a.counts[j] = 0;
    const int64_t nkeys = P.keys[m + 1] - P.keys[m] - 1;
    if (j < nkeys) a.cursor[j] = 0;
    if (j < 2) {
      a.nactive[j] = 0;
      a.outside[j] = 0;
    }
  }
}

__global__ void kr_keys(const RebinArgs *__restrict__ R, RebinPrefix P) {
  const int64_t total = P.pts[P.nmem];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = member_of(P.pts, P.nmem, i);
    const int64_t p = i - P.pts[m];
    const RebinArgs &a = R[m];
    // the cell key of kx_keys
    const double2 up = a.src.u[p];
    int cx = (int)floor(up.x), cy = (int)floor(up.y);
    if (!(up.x >= 0.0 && up.y >= 0.0 && cx < a.nx && cy < a.ny)) {
      atomicOr(a.status, (uint32_t)HG_STATUS_OUT_OF_GRID);
      cx = min(max(cx, 0), a.nx - 1);
      cy = min(max(cy, 0), a.ny - 1);
    }
    const int key = ((cy / BIN) * a.ntx + cx / BIN) * BIN_CELLS + (cy % BIN) * BIN + (cx % BIN);
    a.keys[p] = key;
    atomicAdd(&a.counts[key], 1);
  }
}

// One CTA per (member, chunk): the chunk's sum of counts.
__global__ void __launch_bounds__(THREADS) kr_chunk_sums(const RebinArgs *__restrict__ R,
                                                         RebinPrefix P) {
  const int64_t total = P.chunks[P.nmem];
  for (int64_t blk = blockIdx.x; blk < total; blk += gridDim.x) {
    const int m = member_of(P.chunks, P.nmem, blk);
    const int64_t c = blk - P.chunks[m];
    const int64_t n = P.keys[m + 1] - P.keys[m]; // nkeys + 1
    const RebinArgs &a = R[m];
    int s = 0;
    for (int k = 0; k < RB_CHUNK / THREADS; ++k) {
      const int64_t i = c * RB_CHUNK + k * THREADS + threadIdx.x;
      if (i < n) s += a.counts[i];
    }
    int tot;
    block_excl_scan<THREADS>(s, &tot);
    if (threadIdx.x == 0) a.chunk_sums[c] = tot;
  }
}

// One CTA per member: exclusive scan of its chunk sums, in place.
__global__ void __launch_bounds__(THREADS) kr_chunk_scan(const RebinArgs *__restrict__ R,
                                                         RebinPrefix P) {
  for (int m = blockIdx.x; m < P.nmem; m += gridDim.x) {
    const int64_t nch = P.chunks[m + 1] - P.chunks[m];
    int32_t *cs = R[m].chunk_sums;
    int carry = 0;
    for (int64_t base = 0; base < nch; base += THREADS) {
      const int64_t i = base + threadIdx.x;
      const int v = i < nch ? cs[i] : 0;
      int tot;
      const int ex = block_excl_scan<THREADS>(v, &tot);
      if (i < nch) cs[i] = carry + ex;
      carry += tot;
    }
  }
}

// One CTA per (member, chunk): offsets = exclusive scan of counts.
__global__ void __launch_bounds__(THREADS) kr_chunk_scan_apply(const RebinArgs *__restrict__ R,
                                                               RebinPrefix P) {
  constexpr int ITEMS = RB_CHUNK / THREADS;
  const int64_t total = P.chunks[P.nmem];
  for (int64_t blk = blockIdx.x; blk < total; blk += gridDim.x) {
    const int m = member_of(P.chunks, P.nmem, blk);
    const int64_t c = blk - P.chunks[m];
    const int64_t n = P.keys[m + 1] - P.keys[m];
    const RebinArgs &a = R[m];
    int v[ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const int64_t i = c * RB_CHUNK + (int64_t)threadIdx.x * ITEMS + k;
      v[k] = i < n ? a.counts[i] : 0;
      s += v[k];
    }
    int tot;
    int run = block_excl_scan<THREADS>(s, &tot) + a.chunk_sums[c];
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const int64_t i = c * RB_CHUNK + (int64_t)threadIdx.x * ITEMS + k;
      if (i < n) a.offsets[i] = run;
      run += v[k];
    }
  }
}

__global__ void kr_scatter(const RebinArgs *__restrict__ R, RebinPrefix P) {
  const int64_t total = P.pts[P.nmem];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = member_of(P.pts, P.nmem, i);
    const int64_t p = i - P.pts[m];
    const RebinArgs &a = R[m];
    const int key = a.keys[p];
    const int64_t d = a.offsets[key] + atomicAdd(&a.cursor[key], 1);
    a.dst.u[d] = a.src.u[p];
    a.dst.v[d] = a.src.v[p];
    a.dst.mv[d] = a.src.mv[p];
    a.dst.strain[d] = a.src.strain[p];
    a.dst.flags[d] = a.src.flags[p];
    a.dst.id[d] = a.src.id[p];
    if (a.src.hl) a.dst.hl[d] = a.src.hl[p];
  }
}

__global__ void kr_active(const RebinArgs *__restrict__ R, RebinPrefix P) {
  const int64_t total = P.bins[P.nmem];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = member_of(P.bins, P.nmem, i);
    const int b = (int)(i - P.bins[m]);
    const RebinArgs &a = R[m];
    const int32_t *off = a.offsets;
    auto count = [&](int t) { return off[(t + 1) * BIN_CELLS] - off[t * BIN_CELLS]; };
    if (count(b) > 0) a.bins[atomicAdd(&a.nactive[0], 1)] = b;
    const int tx = b % a.ntx, ty = b / a.ntx;
    bool any = false;
    for (int dy = -1; dy <= 1 && !any; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int x = tx + dx, y = ty + dy;
        if (x < 0 || y < 0 || x >= a.ntx || y >= a.nty) continue;
        if (count(y * a.ntx + x) > 0) {
          any = true;
          break;
        }
      }
    if (any) a.tiles[atomicAdd(&a.nactive[1], 1)] = b;
  }
}

// kx_clear_inactive over (member, tile) items, one block per item
__global__ void __launch_bounds__(BIN_CELLS) kr_clear_inactive(const RebinArgs *__restrict__ R,
                                                               RebinPrefix P) {
  const int64_t total = P.bins[P.nmem];
  for (int64_t i = blockIdx.x; i < total; i += gridDim.x) {
    const int m = member_of(P.bins, P.nmem, i);
    const RebinArgs &a = R[m];
    clear_inactive_tile(a.nx, a.ny, a.ntx, a.nty, a.offsets, (int)(i - P.bins[m]), a.va, a.gm);
  }
}

// ---- upload / download conversion -------------------------------------------

// Elements 2k and 2k + 1 of a: one 16-byte load when a is 16-byte aligned.
__device__ __forceinline__ double2 pair_at(const double *__restrict__ a, int64_t k) {
  if (((uintptr_t)a & 15u) == 0) return reinterpret_cast<const double2 *>(a)[k];
  return make_double2(a[2 * k], a[2 * k + 1]);
}

// Upload index i of the staging arrays (reference layouts) converted into
// slot d of dst; returns the point's position in grid units.
__device__ __forceinline__ double2 upload_point(int64_t i, int64_t d, double gx, double gy,
                                                double h, const double *__restrict__ q,
                                                const double *__restrict__ v,
                                                const double *__restrict__ m,
                                                const double *__restrict__ vol,
                                                const double *__restrict__ hl,
                                                const double *__restrict__ be,
                                                const double *__restrict__ J,
                                                const int32_t *__restrict__ jh,
                                                const uint8_t *__restrict__ kin,
                                                MixedParticles dst) {
  if (dst.hl) dst.hl[d] = (float)(hl[i] / h);
  // pairs read as one 16-byte load where the array allows it (arrays read
  // over the host link arrive in fewer, fuller requests)
  const double2 qq = pair_at(q, i), vv = pair_at(v, i);
  const double2 u = make_double2((qq.x - gx) / h, (qq.y - gy) / h);
  dst.u[d] = u;
  dst.v[d] = make_float2((float)vv.x, (float)vv.y);
  dst.mv[d] = make_float2((float)m[i], (float)vol[i]);
  // absent be, J, jh, kin: the identity, 1, 0 and 0 (a first upload)
  float4 strain = make_float4(0.f, 0.f, 0.f, 0.f);
  if (be) {
    const double2 c0 = pair_at(be, 2 * i), c1 = pair_at(be, 2 * i + 1);
    const double b00 = c0.x, b10 = c0.y, b01 = c1.x, b11 = c1.y;
    strain.y = (float)(b00 - 1.0);
    strain.z = (float)(0.5 * (b10 + b01));
    strain.w = (float)(b11 - 1.0);
  }
  if (J) strain.x = (float)(J[i] - 1.0);
  dst.strain[d] = strain;
  dst.flags[d] = (uint8_t)((jh && jh[i] != 0 ? 1 : 0) | (kin && kin[i] != 0 ? 2 : 0));
  dst.id[d] = (int32_t)i;
  return u;
}

// Upload indices [i0, i1) into the same slots (the re-sort follows).
__global__ void kx_upload(int64_t i0, int64_t i1, double gx, double gy, double h,
                          const double *__restrict__ q, const double *__restrict__ v,
                          const double *__restrict__ m, const double *__restrict__ vol,
                          const double *__restrict__ hl, const double *__restrict__ be,
                          const double *__restrict__ J, const int32_t *__restrict__ jh,
                          const uint8_t *__restrict__ kin, MixedParticles dst) {
  const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= i1) return;
  upload_point(i, i, gx, gy, h, q, v, m, vol, hl, be, J, jh, kin, dst);
}

// Upload indices [i0, i1) into the slots the last re-sort gave them
// (inv); *flag is set when a point is not in the G2P window of its slot's
// tile (skey), or not in the grid: the kernels' tile lists then do not cover
// it and the points must be re-sorted before they are used.
__global__ void kx_upload_slots(int64_t i0, int64_t i1, int64_t n, int nx, int ny, int ntx,
                                double gx, double gy, double h, const double *__restrict__ q,
                                const double *__restrict__ v, const double *__restrict__ m,
                                const double *__restrict__ vol, const double *__restrict__ hl,
                                const double *__restrict__ be, const double *__restrict__ J,
                                const int32_t *__restrict__ jh, const uint8_t *__restrict__ kin,
                                const int32_t *__restrict__ inv,
                                const int32_t *__restrict__ skey, MixedParticles dst,
                                uint32_t *flag) {
  const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= i1) return;
  const int32_t d = inv[i];
  if (d < 0 || d >= n) {
    atomicOr(flag, 1u);
    return;
  }
  const double2 u = upload_point(i, d, gx, gy, h, q, v, m, vol, hl, be, J, jh, kin, dst);
  int cx, cy;
  float fx, fy;
  split_u(u.x, cx, fx);
  split_u(u.y, cy, fy);
  far_edge(nx, cx, fx);
  far_edge(ny, cy, fy);
  const int tile = skey[d] / BIN_CELLS;
  const int wx = cx - ((tile % ntx) * BIN - DRIFT), wy = cy - ((tile / ntx) * BIN - DRIFT);
  const bool in_grid = cx >= 0 && cy >= 0 && cx < nx && cy < ny;
  if (!in_grid || (unsigned)wx > (unsigned)(VA_W - 2) || (unsigned)wy > (unsigned)(VA_W - 2))
    atomicOr(flag, 1u);
}

// Slot k of src into output index o (reference layouts).
__device__ __forceinline__ void download_point(int64_t k, int64_t o, double gx, double gy,
                                               double h, MixedParticles src, double *q,
                                               double *v, double *be, double *J, int32_t *jh) {
  if (q) {
    const double2 u = src.u[k];
    q[2 * o] = gx + u.x * h;
    q[2 * o + 1] = gy + u.y * h;
  }
  if (v) {
    const float2 vv = src.v[k];
    v[2 * o] = vv.x;
    v[2 * o + 1] = vv.y;
  }
  if (be || J) {
    const float4 s = src.strain[k];
    if (be) {
      be[4 * o] = 1.0 + (double)s.y;
      be[4 * o + 1] = (double)s.z;
      be[4 * o + 2] = (double)s.z;
      be[4 * o + 3] = 1.0 + (double)s.w;
    }
    if (J) J[o] = 1.0 + (double)s.x;
  }
  if (jh) jh[o] = src.flags[k] & 1;
}

__global__ void kx_download(int64_t n, double gx, double gy, double h, MixedParticles src,
                            double *q, double *v, double *be, double *J, int32_t *jh) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  download_point(k, src.id[k], gx, gy, h, src, q, v, be, J, jh);
}

// Output indices from the slots inv gives them, 256 per block, written to the
// caller's arrays through shared memory: each warp store then covers whole
// 16-byte pieces of consecutive outputs (over the host link, stores that
// leave parts of a line for a later instruction cost a read-modify-write at
// the host). The arrays must be 16-byte aligned; absent ones are skipped.
__global__ void __launch_bounds__(256) kx_download_lines(int64_t n, double gx, double gy,
                                                         double h, MixedParticles src,
                                                         const int32_t *__restrict__ inv,
                                                         double *q, double *v, double *be,
                                                         double *J, int32_t *jh) {
  __shared__ __align__(16) double s_q[512], s_v[512], s_be[1024], s_J[256];
  __shared__ __align__(16) int32_t s_jh[256];
  const int t = threadIdx.x;
  const int64_t o0 = (int64_t)blockIdx.x * 256;
  const int cnt = (int)(n - o0 < 256 ? n - o0 : 256);
  if (t < cnt) {
    int32_t k = inv[o0 + t];
    if (k < 0 || k >= n) k = 0; // (the order tables cover every upload index)
    const double2 u = src.u[k];
    s_q[2 * t] = gx + u.x * h;
    s_q[2 * t + 1] = gy + u.y * h;
    const float2 vv = src.v[k];
    s_v[2 * t] = vv.x;
    s_v[2 * t + 1] = vv.y;
    const float4 st = src.strain[k];
    s_be[4 * t] = 1.0 + (double)st.y;
    s_be[4 * t + 1] = (double)st.z;
    s_be[4 * t + 2] = (double)st.z;
    s_be[4 * t + 3] = 1.0 + (double)st.w;
    s_J[t] = 1.0 + (double)st.x;
    s_jh[t] = src.flags[k] & 1;
  }
  __syncthreads();
  const double2 *q2 = reinterpret_cast<const double2 *>(s_q);
  const double2 *v2 = reinterpret_cast<const double2 *>(s_v);
  const double2 *b2 = reinterpret_cast<const double2 *>(s_be);
  if (q && t < cnt) reinterpret_cast<double2 *>(q + 2 * o0)[t] = q2[t];
  if (v && t < cnt) reinterpret_cast<double2 *>(v + 2 * o0)[t] = v2[t];
  if (be) {
    double2 *d = reinterpret_cast<double2 *>(be + 4 * o0);
    for (int c = t; c < 2 * cnt; c += 256) d[c] = b2[c];
  }
  if (J) {
    if (2 * t + 1 < cnt) {
      reinterpret_cast<double2 *>(J + o0)[t] = reinterpret_cast<const double2 *>(s_J)[t];
    } else if (2 * t + 1 == cnt) {
      J[o0 + 2 * t] = s_J[2 * t];
    }
  }
  if (jh) {
    if (4 * t + 3 < cnt) {
      reinterpret_cast<int4 *>(jh + o0)[t] = reinterpret_cast<const int4 *>(s_jh)[t];
    } else {
      for (int c = 4 * t; c < cnt && c < 4 * t + 4; ++c) jh[o0 + c] = s_jh[c];
    }
  }
}


__global__ void kx_grid_download(int64_t nn, const float *__restrict__ gm,
                                 const float4 *__restrict__ va, double *mass, double *vel,
                                 double *acc) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const float4 a = va[i];
  mass[i] = gm[i];
  vel[2 * i] = a.x;
  vel[2 * i + 1] = a.y;
  acc[2 * i] = a.z;
  acc[2 * i + 1] = a.w;
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

MixedParticles parts(hg_mpm *m, int which) {
  MixedParticles P;
  P.u = m->mu_[which].p;
  P.v = m->mv_[which].p;
  P.mv = m->mmv_[which].p;
  P.strain = m->mstrain_[which].p;
  P.flags = m->mflags_[which].p;
  P.id = m->mid_[which].p;
  P.hl = m->mhl_[which].p; // nullptr for the linear basis
  return P;
}

size_t fused_smem_bytes() { return 0; } // static shared memory only

MixedArgs make_args(hg_mpm *m, double dt, bool tiles) {
  MixedArgs A;
  const hg::MpmParams &P = m->p;
  A.nx = P.nx;
  A.ny = P.ny;
  A.ntx = m->ntx;
  A.nty = m->nty;
  A.n = m->n;
  A.gmin[0] = P.gmin[0];
  A.gmin[1] = P.gmin[1];
  A.h = P.h;
  A.dt = (float)dt;
  A.inv_h = (float)P.inv_h;
  A.kappa = (float)P.kappa;
  A.mu = (float)P.mu;
  A.dp_alpha = (float)P.dp_alpha;
  A.flip_alpha = (float)P.flip_alpha;
  A.gx = (float)P.g[0];
  A.gy = (float)P.g[1];
  A.pmargin = 0.01f + 4.0e-7f * (float)(P.nx + P.ny);
  A.nplanes = P.nplanes;
  for (int k = 0; k < HG_MAX_PLANES; ++k) A.planes[k] = P.planes[k];
  A.offsets = m->offsets.p;
  A.active = tiles ? m->active_tiles.p : m->active_bins.p;
  A.nactive = tiles ? m->nactive.p + 1 : m->nactive.p;
  MixedParticles cur = parts(m, m->cur);
  A.u = cur.u;
  A.v = cur.v;
  A.mv = cur.mv;
  A.strain = cur.strain;
  A.flags = cur.flags;
  A.hl = cur.hl;
  A.va = m->va.p;
  A.va_out = m->va.p;
  A.acc4 = m->acc4.p;
  A.accm = m->accm.p;
  A.gm = m->gm.p;
  A.status = m->status.p;
  A.outside = m->outside.p;
  return A;
}

hg_status rebin(hg_mpm *m) {
  cudaStream_t s = m->ctx->stream;
  const int64_t nkeys = (int64_t)m->ntx * m->nty * BIN_CELLS;
  HG_CUDA_TRY(cudaMemsetAsync(m->counts.p, 0, sizeof(int32_t) * (nkeys + 1), s));
  HG_CUDA_TRY(cudaMemsetAsync(m->cursor.p, 0, sizeof(int32_t) * nkeys, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->nactive.p, 0, sizeof(int32_t) * 2, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->outside.p, 0, 2 * sizeof(uint32_t), s));
  if (m->n > 0) {
    HG_LAUNCH(kx_keys, blocks_for(m->n, 256), 256, 0, s, m->n, m->p.nx, m->p.ny, m->ntx,
              m->mu_[m->cur].p, m->keys.p, m->counts.p, m->status.p);
    HG_CHECK_LAUNCH();
  }
  hg_status st = exclusive_scan_i32(m->counts.p, m->offsets.p, nkeys + 1, m->scan_tmp.p, s);
  if (st != HG_OK) return st;
  if (m->n > 0) {
    HG_LAUNCH(kx_scatter, blocks_for(m->n, 256), 256, 0, s, m->n, m->keys.p, m->offsets.p,
              m->cursor.p, parts(m, m->cur), parts(m, 1 - m->cur), m->inv.p, m->skey.p);
    HG_CHECK_LAUNCH();
  }
  m->cur = 1 - m->cur;
  m->order_valid = true;
  m->order_n = m->n;
  HG_LAUNCH(kx_active, blocks_for((int64_t)m->ntx * m->nty, 256), 256, 0, s, m->ntx, m->nty,
            m->offsets.p, m->active_bins.p, m->active_tiles.p, m->nactive.p);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kx_clear_inactive, std::min(m->ntx * m->nty, m->ctx->num_sms * 8), BIN_CELLS, 0, s,
            m->p.nx, m->p.ny, m->ntx, m->nty, m->offsets.p, m->va.p, m->gm.p);
  HG_CHECK_LAUNCH();
  m->steps_since_rebin = 0;
  m->outside_pending = false;
  m->rebins++;
  return HG_OK;
}

// Space for the batched re-sort's argument table of up to nmax members.
size_t rebin_table_bytes(int nmax) {
  return (size_t)nmax * sizeof(RebinArgs) + 4 * (size_t)(nmax + 1) * sizeof(int64_t);
}

// Re-sorts the given members in eight launches. table: page-locked host staging
// (rebin_table_bytes), dtable: its device copy; both free to overwrite.
hg_status rebin_batch(hg_context *ctx, const std::vector<hg_mpm *> &R, unsigned char *table,
                      unsigned char *dtable) {
  cudaStream_t s = ctx->stream;
  const int nm = (int)R.size();
  RebinArgs *args = reinterpret_cast<RebinArgs *>(table);
  int64_t *pre = reinterpret_cast<int64_t *>(table + (size_t)nm * sizeof(RebinArgs));
  int64_t *pp = pre, *pk = pre + (nm + 1), *pc = pre + 2 * (nm + 1), *pb = pre + 3 * (nm + 1);
  pp[0] = pk[0] = pc[0] = pb[0] = 0;
  int64_t max_items = 0;
  for (int i = 0; i < nm; ++i) {
    hg_mpm *m = R[i];
    const int64_t nkeys = (int64_t)m->ntx * m->nty * BIN_CELLS;
    RebinArgs &a = args[i];
    a.n = m->n;
    a.nx = m->p.nx;
    a.ny = m->p.ny;
    a.ntx = m->ntx;
    a.nty = m->nty;
    a.src = parts(m, m->cur);
    a.dst = parts(m, 1 - m->cur);
    a.keys = m->keys.p;
    a.counts = m->counts.p;
    a.offsets = m->offsets.p;
    a.cursor = m->cursor.p;
    a.bins = m->active_bins.p;
    a.tiles = m->active_tiles.p;
    a.nactive = m->nactive.p;
    a.chunk_sums = m->scan_tmp.p;
    a.status = m->status.p;
    a.outside = m->outside.p;
    a.va = m->va.p;
    a.gm = m->gm.p;
    pp[i + 1] = pp[i] + m->n;
    pk[i + 1] = pk[i] + nkeys + 1;
    pc[i + 1] = pc[i] + (nkeys + 1 + RB_CHUNK - 1) / RB_CHUNK;
    pb[i + 1] = pb[i] + (int64_t)m->ntx * m->nty;
    max_items = std::max(max_items, std::max(pp[i + 1], pk[i + 1]));
  }
  const size_t bytes = (size_t)nm * sizeof(RebinArgs) + 4 * (size_t)(nm + 1) * sizeof(int64_t);
  HG_CUDA_TRY(cudaMemcpyAsync(dtable, table, bytes, cudaMemcpyHostToDevice, s));
  const RebinArgs *dR = reinterpret_cast<const RebinArgs *>(dtable);
  const int64_t *dpre = reinterpret_cast<const int64_t *>(dtable + (size_t)nm * sizeof(RebinArgs));
  RebinPrefix P{dpre, dpre + (nm + 1), dpre + 2 * (nm + 1), dpre + 3 * (nm + 1), nm};
  const int cap = ctx->num_sms * 8;
  auto grid = [&](int64_t items) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(cap, (items + 255) / 256));
  };
  HG_LAUNCH(kr_clear, grid(pk[nm]), 256, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_keys, grid(pp[nm]), 256, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  const int cgrid = (int)std::min<int64_t>(pc[nm], (int64_t)ctx->num_sms * 8);
  HG_LAUNCH(kr_chunk_sums, cgrid, THREADS, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_chunk_scan, nm, THREADS, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_chunk_scan_apply, cgrid, THREADS, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_scatter, grid(pp[nm]), 256, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_active, grid(pb[nm]), 256, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  HG_LAUNCH(kr_clear_inactive, (int)std::max<int64_t>(1, std::min<int64_t>(pb[nm], cap)),
            BIN_CELLS, 0, s, dR, P);
  HG_CHECK_LAUNCH();
  for (hg_mpm *m : R) {
    m->cur = 1 - m->cur;
    m->order_valid = false; // the batched re-sort keeps no order tables
    m->steps_since_rebin = 0;
    m->outside_pending = false;
    m->rebins++;
  }
  return HG_OK;
}

// CTAs per SM of the two kernels: the launch shape, else 3 (the fused
// kernel's occupancy at 80 registers) and 8
constexpr int DEFAULT_FUSED_CTAS = 3, DEFAULT_UPDATE_CTAS = 8;
int fused_per_sm(const hg_launch_shape &s) {
  return s.fused_ctas_per_sm > 0 ? s.fused_ctas_per_sm : DEFAULT_FUSED_CTAS;
}
int update_per_sm(const hg_launch_shape &s) {
  return s.update_ctas_per_sm > 0 ? s.update_ctas_per_sm : DEFAULT_UPDATE_CTAS;
}
int fused_blocks(hg_mpm *m) { return m->ctx->num_sms * fused_per_sm(m->shape); }
// the uGIMP kernel walks the points: up to 8 CTAs per SM
int ugimp_blocks(hg_mpm *m) {
  const int64_t b = (m->n + THREADS - 1) / THREADS;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)m->ctx->num_sms * 8));
}
// G2P of this step fused with P2G of the next (or the first P2G, PRIME)
template <bool PRIME>
void launch_particle_kernel(hg_mpm *m, const MixedArgs &A, cudaStream_t s) {
  if (m->p.basis == HG_BASIS_UGIMP) {
    HG_LAUNCH_PDL(kxu_step<PRIME>, ugimp_blocks(m), THREADS, 0, s, A);
  } else {
    HG_LAUNCH_PDL(kx_g2p2g<PRIME>, fused_blocks(m), THREADS, fused_smem_bytes(), s, A);
  }
}
int update_blocks(hg_mpm *m) { return m->ctx->num_sms * update_per_sm(m->shape); }
bool same_shape(const hg_launch_shape &a, const hg_launch_shape &b) {
  return a.fused_ctas_per_sm == b.fused_ctas_per_sm &&
         a.update_ctas_per_sm == b.update_ctas_per_sm;
}

// ---- the tuning table -------------------------------------------------------
//
// Keyed by (kind, SMs, tiles, points), tiles and points rounded up to powers
// of two: kind 0 is a single scene, kind 1 a batch (tiles 0).
using TuneKey = std::array<int64_t, 4>;
std::mutex g_tune_mu;
std::map<TuneKey, hg_launch_shape> g_tune;

int64_t ceil_pow2(int64_t x) {
  int64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
TuneKey mixed_key(const hg_mpm *m) {
  return {0, m->ctx->num_sms, ceil_pow2((int64_t)m->ntx * m->nty), ceil_pow2(std::max<int64_t>(m->n, 1))};
}
TuneKey batch_key(const hg_batch *b, int64_t points) {
  return {1, b->ctx->num_sms, 0, ceil_pow2(std::max<int64_t>(points, 1))};
}
bool tune_lookup(const TuneKey &k, hg_launch_shape *out) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(k);
  if (it == g_tune.end()) return false;
  *out = it->second;
  return true;
}
void tune_store(const TuneKey &k, const hg_launch_shape &s) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[k] = s;
}
// CTAs per SM tried for (fused, update): fewer, the default, and more CTAs
// than are resident (finer shares of the tiles, later ones fill in behind
// the first wave)
constexpr hg_launch_shape TUNE_CANDIDATES[HG_TUNE_CANDIDATES] = {{2, 4}, {3, 8}, {6, 16},
                                                                 {12, 32}};
static_assert(HG_TUNE_CANDIDATES == 4, "candidate list");

hg_status prime(hg_mpm *m) {
  cudaStream_t s = m->ctx->stream;
  if (!m->shape_set && !tune_lookup(mixed_key(m), &m->shape)) m->shape = hg_launch_shape{0, 0};
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  HG_CUDA_TRY(cudaMemsetAsync(m->accm.p, 0, sizeof(float) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->acc4.p, 0, sizeof(float4) * nn, s));
  hg_status st = rebin(m);
  if (st != HG_OK) return st;
  MixedArgs A = make_args(m, 0.0, false);
  launch_particle_kernel<true>(m, A, s);
  HG_CHECK_LAUNCH();
  m->primed = true;
  return HG_OK;
}

} // namespace

hg_status mixed_alloc(hg_mpm *m) {
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  m->ntx = (m->p.nx + 1 + BIN - 1) / BIN;
  m->nty = (m->p.ny + 1 + BIN - 1) / BIN;
  const int64_t nkeys = (int64_t)m->ntx * m->nty * BIN_CELLS;
  if (nkeys + 1 > (int64_t)INT32_MAX / 2)
    return fail(HG_ERR_INVALID_ARGUMENT, "grid too large for the MIXED path");
  for (int b = 0; b < 2; ++b) {
    hg_status st;
    if ((st = m->mu_[b].alloc(m->cap)) || (st = m->mv_[b].alloc(m->cap)) ||
        (st = m->mmv_[b].alloc(m->cap)) || (st = m->mstrain_[b].alloc(m->cap)) ||
        (st = m->mflags_[b].alloc(m->cap)) || (st = m->mid_[b].alloc(m->cap)))
      return st;
    if (m->p.basis == HG_BASIS_UGIMP && (st = m->mhl_[b].alloc(m->cap))) return st;
  }
  hg_status st;
  if ((st = m->acc4.alloc(nn)) || (st = m->accm.alloc(nn)) || (st = m->va.alloc(nn)) ||
      (st = m->gm.alloc(nn)) || (st = m->keys.alloc(m->cap)) ||
      (st = m->counts.alloc(nkeys + 1)) || (st = m->offsets.alloc(nkeys + 1)) ||
      (st = m->cursor.alloc(nkeys)) || (st = m->scan_tmp.alloc(scan_tmp_size(nkeys + 1))) ||
      (st = m->active_bins.alloc((int64_t)m->ntx * m->nty)) ||
      (st = m->active_tiles.alloc((int64_t)m->ntx * m->nty)) ||
      (st = m->nactive.alloc(2)) || (st = m->outside.alloc(2)))
    return st;
  cudaStream_t s = m->ctx->stream;
  HG_CUDA_TRY(cudaMemsetAsync(m->acc4.p, 0, sizeof(float4) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->accm.p, 0, sizeof(float) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->va.p, 0, sizeof(float4) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->gm.p, 0, sizeof(float) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->nactive.p, 0, sizeof(int32_t) * 2, s));
  if ((st = m->inv.alloc(m->cap)) || (st = m->skey.alloc(m->cap)) || (st = m->d_flag.alloc(1)))
    return st;
  m->h_outside = context_pinned_pair(m->ctx);
  m->h_flag = context_pinned_pair(m->ctx);
  if (!m->h_outside || !m->h_flag) return fail(HG_ERR_OUT_OF_MEMORY, "page-locked host memory");
  m->h_outside[0] = m->h_outside[1] = 0;
  HG_CUDA_TRY(cudaEventCreateWithFlags(&m->outside_ev, cudaEventDisableTiming));
  return HG_OK;
}

int64_t mixed_device_bytes(int nx, int ny, int64_t cap) {
  const int64_t nn = (int64_t)(nx + 1) * (ny + 1);
  const int64_t ntx = (nx + 1 + BIN - 1) / BIN, nty = (ny + 1 + BIN - 1) / BIN;
  const int64_t nkeys = ntx * nty * BIN_CELLS;
  const int64_t per_point = sizeof(double2) + 2 * sizeof(float2) + sizeof(float4) + 1 + 4;
  int64_t b = 2 * cap * per_point + cap * 4 * 3;             // particle pairs, keys, order tables
  b += nn * (2 * sizeof(float4) + 2 * sizeof(float));       // acc4, va, accm, gm
  b += 4 * (3 * nkeys + 2 + scan_tmp_size(nkeys + 1));      // counts, offsets, cursor
  b += 4 * (2 * ntx * nty + 4);                             // active lists, counters
  return b;
}

hg_status mixed_upload(hg_mpm *m, const double *q, const double *v, const double *mass,
                       const double *vol, const double *hl, const double *be, const double *J,
                       const int32_t *jh, const uint8_t *kin) {
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  if (m->p.basis == HG_BASIS_UGIMP && n > 0 && !hl)
    return fail(HG_ERR_INVALID_ARGUMENT, "the uGIMP basis needs the half-widths hl");
  if (n > 0) {
    HG_LAUNCH(kx_upload, blocks_for(n, 256), 256, 0, s, (int64_t)0, n, m->p.gmin[0],
              m->p.gmin[1], m->p.h, q, v, mass, vol, hl, be, J, jh, kin, parts(m, m->cur));
    HG_CHECK_LAUNCH();
  }
  return prime(m);
}

hg_status mixed_download(hg_mpm *m, double *q, double *v, double *be, double *J, int32_t *jh) {
  if (m->n <= 0) return HG_OK;
  HG_LAUNCH(kx_download, blocks_for(m->n, 256), 256, 0, m->ctx->stream, m->n, m->p.gmin[0],
            m->p.gmin[1], m->p.h, parts(m, m->cur), q, v, be, J, jh);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

namespace {
// The first P2G of points already in the live buffer's sorted order.
hg_status prime_in_order(hg_mpm *m) {
  cudaStream_t s = m->ctx->stream;
  if (!m->shape_set && !tune_lookup(mixed_key(m), &m->shape)) m->shape = hg_launch_shape{0, 0};
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  HG_CUDA_TRY(cudaMemsetAsync(m->accm.p, 0, sizeof(float) * nn, s));
  HG_CUDA_TRY(cudaMemsetAsync(m->acc4.p, 0, sizeof(float4) * nn, s));
  MixedArgs A = make_args(m, 0.0, false);
  launch_particle_kernel<true>(m, A, s);
  HG_CHECK_LAUNCH();
  m->primed = true;
  return HG_OK;
}
} // namespace

hg_status mixed_upload_direct(hg_mpm *m, const double *q, const double *v, const double *mass,
                              const double *vol, const double *hl, const double *be,
                              const double *J, const int32_t *jh, const uint8_t *kin) {
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  if (m->p.basis == HG_BASIS_UGIMP && n > 0 && !hl)
    return fail(HG_ERR_INVALID_ARGUMENT, "the uGIMP basis needs the half-widths hl");
  const MixedParticles dst = parts(m, m->cur);
  const double gx = m->p.gmin[0], gy = m->p.gmin[1], h = m->p.h;
  hg_status st;
  // the points keep the slots of the last re-sort when it sorted this many
  if (n > 0 && m->order_valid && m->order_n == n) {
    HG_CUDA_TRY(cudaMemsetAsync(m->d_flag.p, 0, sizeof(uint32_t), s));
    HG_LAUNCH(kx_upload_slots, blocks_for(n, 256), 256, 0, s, (int64_t)0, n, n, m->p.nx,
              m->p.ny, m->ntx, gx, gy, h, q, v, mass, vol, hl, be, J, jh, kin, m->inv.p,
              m->skey.p, dst, m->d_flag.p);
    HG_CHECK_LAUNCH();
    HG_CUDA_TRY(cudaMemcpyAsync(m->h_flag, m->d_flag.p, sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, s));
    if ((st = prime_in_order(m))) return st;
    HG_CUDA_TRY(cudaStreamSynchronize(s));
    if (m->h_flag[0] == 0) return HG_OK;
    m->primed = false; // a point left its slot's window: a first upload follows
  }
  if (n > 0) {
    HG_LAUNCH(kx_upload, blocks_for(n, 256), 256, 0, s, (int64_t)0, n, gx, gy, h, q, v, mass,
              vol, hl, be, J, jh, kin, dst);
    HG_CHECK_LAUNCH();
  }
  if ((st = prime(m))) return st;
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status mixed_download_direct(hg_mpm *m, double *q, double *v, double *be, double *J,
                                int32_t *jh, bool *done) {
  *done = false;
  const int64_t n = m->n;
  if (n <= 0 || !m->order_valid || m->order_n != n) return HG_OK;
  HG_LAUNCH(kx_download_lines, blocks_for(n, 256), 256, 0, m->ctx->stream, n, m->p.gmin[0],
            m->p.gmin[1], m->p.h, parts(m, m->cur), m->inv.p, q, v, be, J, jh);
  HG_CHECK_LAUNCH();
  *done = true;
  return HG_OK;
}

hg_status mixed_download_grid(hg_mpm *m, double *mass, double *vel, double *acc) {
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  HG_LAUNCH(kx_grid_download, blocks_for(nn, 256), 256, 0, m->ctx->stream, nn, m->gm.p,
            m->va.p, mass, vel, acc);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

// Maximum number of steps between two re-sorts. Particles outside their
// window are exact but slow; this bound keeps every particle well inside the
// dilated tile set that the grid update covers.
constexpr int64_t MAX_STEPS_BETWEEN_REBINS = 64;

hg_status mixed_profile_read(hg_mpm *m, double *g2p2g_ms, double *update_ms, int64_t *steps) {
  double a = 0.0, b = 0.0;
  if (m->prof_used > 0) HG_CUDA_TRY(cudaEventSynchronize(m->prof_events[m->prof_used - 1]));
  for (size_t k = 0; k + 2 < m->prof_used; k += 3) {
    float t01 = 0.f, t12 = 0.f;
    HG_CUDA_TRY(cudaEventElapsedTime(&t01, m->prof_events[k], m->prof_events[k + 1]));
    HG_CUDA_TRY(cudaEventElapsedTime(&t12, m->prof_events[k + 1], m->prof_events[k + 2]));
    b += t01;
    a += t12;
  }
  if (g2p2g_ms) *g2p2g_ms = a;
  if (update_ms) *update_ms = b;
  if (steps) *steps = (int64_t)(m->prof_used / 3);
  return HG_OK;
}

// Steps per captured chunk. Re-sort decisions are taken between chunks; the
// cadence only affects speed (points outside their window stay exact), and
// at a CFL number below 1 no point crosses a tile within a chunk.
constexpr int CHUNK_STEPS = 16;

// Ends a capture begun on s, restoring the launch counter that the captured
// launches advanced; instantiates the graph into *exec and returns the
// number of kernel launches one replay performs.
hg_status end_chunk_capture(cudaStream_t s, hg_status st, int64_t l0, cudaGraphExec_t *exec,
                            int64_t *launches) {
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  *launches = g_launches.load() - l0;
  g_launches.fetch_sub(*launches, std::memory_order_relaxed);
  if (st != HG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  const cudaError_t ei = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    *exec = nullptr;
    return cuda_fail(ei, "cudaGraphInstantiate");
  }
  return HG_OK;
}

// The graph of CHUNK_STEPS steps of one scene for its live buffer: the two
// kernels per step, then the read-back of the out-of-window counters.
hg_status mixed_chunk_graph(hg_mpm *m, double dt) {
  const int c = m->cur;
  if (m->chunk_exec[c] && m->chunk_dt[c] == dt && m->chunk_n[c] == m->n &&
      same_shape(m->chunk_shape[c], m->shape))
    return HG_OK;
  if (m->chunk_exec[c]) {
    cudaGraphExecDestroy(m->chunk_exec[c]);
    m->chunk_exec[c] = nullptr;
  }
  cudaStream_t s = m->ctx->stream;
  const size_t smem = fused_smem_bytes();
  const MixedArgs At = make_args(m, dt, true), Ab = make_args(m, dt, false);
  const int64_t l0 = g_launches.load();
  HG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  hg_status st = HG_OK;
  for (int k = 0; k < CHUNK_STEPS && st == HG_OK; ++k) {
    HG_LAUNCH_PDL(kx_grid_update, update_blocks(m), THREADS, 0, s, At);
    launch_particle_kernel<false>(m, Ab, s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_fail(e, "kernel launch");
  }
  if (st == HG_OK) {
    const cudaError_t e = cudaMemcpyAsync(m->h_outside, m->outside.p, 2 * sizeof(uint32_t),
                                          cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync");
  }
  int64_t launches = 0;
  st = end_chunk_capture(s, st, l0, &m->chunk_exec[c], &launches);
  if (st != HG_OK) return st;
  m->chunk_dt[c] = dt;
  m->chunk_n[c] = m->n;
  m->chunk_shape[c] = m->shape;
  m->chunk_launches = launches;
  return HG_OK;
}

hg_status mixed_step(hg_mpm *m, double dt, int nsteps) {
  cudaStream_t s = m->ctx->stream;
  if (!m->primed) {
    hg_status st = prime(m);
    if (st != HG_OK) return st;
  }
  const size_t smem = fused_smem_bytes();
  int k = 0;
  // whole chunks replay a captured graph (one launch for 2 x CHUNK_STEPS
  // kernels); event timing needs the per-step path
  while (!m->profile && nsteps - k >= CHUNK_STEPS) {
    bool need = m->steps_since_rebin >= MAX_STEPS_BETWEEN_REBINS;
    if (!need && m->outside_pending && cudaEventQuery(m->outside_ev) == cudaSuccess) {
      m->outside_pending = false;
      need = m->h_outside[0] > 0 || (int64_t)m->h_outside[1] * 32 > m->n;
    }
    if (need) {
      hg_status st = rebin(m);
      if (st != HG_OK) return st;
    }
    hg_status st = mixed_chunk_graph(m, dt);
    if (st != HG_OK) return st;
    HG_CUDA_TRY(cudaGraphLaunch(m->chunk_exec[m->cur], s));
    g_launches.fetch_add(m->chunk_launches, std::memory_order_relaxed);
    HG_CUDA_TRY(cudaEventRecord(m->outside_ev, s));
    m->outside_pending = true;
    m->steps_since_rebin += CHUNK_STEPS;
    k += CHUNK_STEPS;
  }
  for (; k < nsteps; ++k) {
    bool need = m->steps_since_rebin >= MAX_STEPS_BETWEEN_REBINS;
    if (!need && m->outside_pending && cudaEventQuery(m->outside_ev) == cudaSuccess) {
      m->outside_pending = false;
      need = m->h_outside[0] > 0 || (int64_t)m->h_outside[1] * 32 > m->n;
    }
    if (need) {
      hg_status st = rebin(m);
      if (st != HG_OK) return st;
    }
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    if (m->profile) {
      while (m->prof_events.size() < m->prof_used + 3) {
        cudaEvent_t e;
        HG_CUDA_TRY(cudaEventCreate(&e));
        m->prof_events.push_back(e);
      }
      for (int j = 0; j < 3; ++j) ev[j] = m->prof_events[m->prof_used + j];
      m->prof_used += 3;
      HG_CUDA_TRY(cudaEventRecord(ev[0], s));
    }
    MixedArgs At = make_args(m, dt, true);
    HG_LAUNCH_PDL(kx_grid_update, update_blocks(m), THREADS, 0, s, At);
    HG_CHECK_LAUNCH();
    if (m->profile) HG_CUDA_TRY(cudaEventRecord(ev[1], s));
    MixedArgs Ab = make_args(m, dt, false);
    launch_particle_kernel<false>(m, Ab, s);
    HG_CHECK_LAUNCH();
    if (m->profile) HG_CUDA_TRY(cudaEventRecord(ev[2], s));
    m->steps_since_rebin++;
    if (!m->outside_pending) {
      HG_CUDA_TRY(cudaMemcpyAsync(m->h_outside, m->outside.p, 2 * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, s));
      HG_CUDA_TRY(cudaEventRecord(m->outside_ev, s));
      m->outside_pending = true;
    }
  }
  return HG_OK;
}

// The per-step body of mixed_step in three parts, for the hybrid step.
hg_status mixed_step_begin(hg_mpm *m) {
  if (!m->primed) {
    hg_status st = prime(m);
    if (st != HG_OK) return st;
  }
  bool need = m->steps_since_rebin >= MAX_STEPS_BETWEEN_REBINS;
  if (!need && m->outside_pending && cudaEventQuery(m->outside_ev) == cudaSuccess) {
    m->outside_pending = false;
    need = m->h_outside[0] > 0 || (int64_t)m->h_outside[1] * 32 > m->n;
  }
  return need ? rebin(m) : HG_OK;
}

hg_status mixed_grid_update(hg_mpm *m, double dt) {
  MixedArgs A = make_args(m, dt, true);
  HG_LAUNCH_PDL(kx_grid_update, update_blocks(m), THREADS, 0, m->ctx->stream, A);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

hg_status mixed_particles(hg_mpm *m, double dt) {
  cudaStream_t s = m->ctx->stream;
  MixedArgs A = make_args(m, dt, false);
  launch_particle_kernel<false>(m, A, s);
  HG_CHECK_LAUNCH();
  m->steps_since_rebin++;
  if (!m->outside_pending) {
    HG_CUDA_TRY(cudaMemcpyAsync(m->h_outside, m->outside.p, 2 * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, s));
    HG_CUDA_TRY(cudaEventRecord(m->outside_ev, s));
    m->outside_pending = true;
  }
  return HG_OK;
}

} // namespace hg

// ---- batches ---------------------------------------------------------------------

namespace hg {

hg_status batch_alloc(hg_batch *b) {
  const size_t tsz = 2 * (size_t)b->max_members * sizeof(MixedArgs);
  hg_status st;
  if ((st = b->table.alloc(tsz)) || (st = b->outside.alloc(2 * (size_t)b->max_members)) ||
      (st = b->queue.alloc(4)))
    return st;
  HG_CUDA_TRY(cudaMemsetAsync(b->queue.p, 0, 4 * sizeof(int32_t), b->ctx->stream));
  for (int k = 0; k < hg_batch::NBUF; ++k) {
    HG_CUDA_TRY(cudaMallocHost(&b->h_table[k], tsz));
    HG_CUDA_TRY(cudaEventCreateWithFlags(&b->table_ev[k], cudaEventDisableTiming));
  }
  b->args.resize(2 * (size_t)b->max_members * sizeof(MixedArgs));
  const size_t rsz = rebin_table_bytes(b->max_members);
  if ((st = b->rtable.alloc(rsz))) return st;
  for (int k = 0; k < hg_batch::NBUF; ++k) {
    HG_CUDA_TRY(cudaMallocHost(&b->h_rtable[k], rsz));
    HG_CUDA_TRY(cudaEventCreateWithFlags(&b->rtable_ev[k], cudaEventDisableTiming));
  }
  HG_CUDA_TRY(cudaMallocHost(&b->h_outside, 2 * sizeof(uint32_t) * b->max_members));
  HG_CUDA_TRY(cudaEventCreateWithFlags(&b->out_ev, cudaEventDisableTiming));
  return HG_OK;
}

void batch_free(hg_batch *b) {
  for (int k = 0; k < hg_batch::NBUF; ++k) {
    if (b->h_table[k]) cudaFreeHost(b->h_table[k]);
    if (b->table_ev[k]) cudaEventDestroy(b->table_ev[k]);
    if (b->h_rtable[k]) cudaFreeHost(b->h_rtable[k]);
    if (b->rtable_ev[k]) cudaEventDestroy(b->rtable_ev[k]);
  }
  if (b->h_outside) cudaFreeHost(b->h_outside);
  if (b->out_ev) cudaEventDestroy(b->out_ev);
  if (b->chunk_exec) cudaGraphExecDestroy(b->chunk_exec);
  for (cudaEvent_t e : b->prof_events) cudaEventDestroy(e);
}

hg_status batch_profile_read(hg_batch *b, double *ms, int64_t *steps) {
  double acc[hg_batch::PROF_PHASES] = {0.0};
  const size_t per = hg_batch::PROF_PHASES + 1;
  if (b->prof_used > 0) HG_CUDA_TRY(cudaEventSynchronize(b->prof_events[b->prof_used - 1]));
  for (size_t k = 0; k + per <= b->prof_used; k += per)
    for (int j = 0; j < hg_batch::PROF_PHASES; ++j) {
      float t = 0.f;
      HG_CUDA_TRY(cudaEventElapsedTime(&t, b->prof_events[k + j], b->prof_events[k + j + 1]));
      acc[j] += t;
    }
  for (int j = 0; j < hg_batch::PROF_PHASES; ++j) ms[j] = acc[j];
  if (steps) *steps = (int64_t)(b->prof_used / per);
  return HG_OK;
}

// The graph of CHUNK_STEPS steps of all S members: the two batched kernels
// per step, then the gather and read-back of the out-of-window counters.
hg_status batch_chunk_graph(hg_batch *b, int S) {
  if (b->chunk_exec && b->chunk_members == S && same_shape(b->chunk_shape, b->shape))
    return HG_OK;
  if (b->chunk_exec) {
    cudaGraphExecDestroy(b->chunk_exec);
    b->chunk_exec = nullptr;
  }
  cudaStream_t s = b->ctx->stream;
  const MixedArgs *dt = reinterpret_cast<const MixedArgs *>(b->table.p);
  const MixedArgs *db = dt + S;
  const int nsm = b->ctx->num_sms;
  const int gu = nsm * update_per_sm(b->shape), gf = nsm * fused_per_sm(b->shape);
  const int64_t l0 = g_launches.load();
  HG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  hg_status st = HG_OK;
  for (int k = 0; k < CHUNK_STEPS && st == HG_OK; ++k) {
    HG_LAUNCH(kb_grid_update, gu, THREADS, 0, s, dt, S, b->queue.p + 2);
    HG_LAUNCH(kb_g2p2g, gf, THREADS, 0, s, db, S, b->queue.p);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_fail(e, "kernel launch");
  }
  if (st == HG_OK) {
    HG_LAUNCH(kb_gather_outside, (S + 127) / 128, 128, 0, s, db, S, b->outside.p);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->h_outside, b->outside.p, 2 * sizeof(uint32_t) * S,
                          cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) st = cuda_fail(e, "chunk capture");
  }
  int64_t launches = 0;
  st = end_chunk_capture(s, st, l0, &b->chunk_exec, &launches);
  if (st != HG_OK) return st;
  b->chunk_members = S;
  b->chunk_shape = b->shape;
  b->chunk_launches = launches;
  return HG_OK;
}

hg_status batch_step(hg_batch *b, int nsteps) {
  cudaStream_t s = b->ctx->stream;
  const int S = (int)b->members.size();
  if (S == 0) return HG_OK;
  MixedArgs *cache = reinterpret_cast<MixedArgs *>(b->args.data());
  if ((int)b->sigs.size() != S) {
    b->sigs.assign(S, hg_batch::Sig{});
    b->dirty = true;
  }
  if (!b->shape_set) {
    int64_t points = 0;
    for (hg_mpm *m : b->members) points += m->n;
    const TuneKey key = batch_key(b, points);
    if (key[3] != b->shape_class) {
      b->shape_class = key[3];
      if (!tune_lookup(key, &b->shape)) b->shape = hg_launch_shape{0, 0};
    }
  }
  // Host work ahead of a step (or of a captured chunk of steps): re-sort
  // members whose points left their windows (counters read back
  // asynchronously), members due for a periodic re-sort and members not yet
  // primed; then bring the argument table up to date.
  auto prepare = [&](cudaEvent_t ev1, cudaEvent_t ev2) -> hg_status {
    if (b->out_pending && cudaEventQuery(b->out_ev) == cudaSuccess) {
      b->out_pending = false;
      for (size_t i = 0; i < b->out_members.size(); ++i) {
        hg_mpm *m = b->out_members[i];
        if (!m) continue;
        if (b->h_outside[2 * i] > 0 || (int64_t)b->h_outside[2 * i + 1] * 32 > m->n)
          m->steps_since_rebin = MAX_STEPS_BETWEEN_REBINS;
      }
    }
    b->due.clear();
    for (hg_mpm *m : b->members) {
      if (!m->primed) {
        const hg_status st = prime(m);
        if (st != HG_OK) return st;
      } else if (m->steps_since_rebin >= MAX_STEPS_BETWEEN_REBINS) {
        b->due.push_back(m);
      }
    }
    if (!b->due.empty()) {
      // the staging buffer last used NBUF re-sorts ago must have been copied
      const int rb = b->rb;
      b->rb = (b->rb + 1) % hg_batch::NBUF;
      const auto w0 = std::chrono::steady_clock::now();
      HG_CUDA_TRY(cudaEventSynchronize(b->rtable_ev[rb]));
      b->wait_ms +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
      // the device table is reused: its previous copy was read by kernels
      // that precede this copy on the stream
      const hg_status st = rebin_batch(b->ctx, b->due, b->h_rtable[rb], b->rtable.p);
      if (st != HG_OK) return st;
      HG_CUDA_TRY(cudaEventRecord(b->rtable_ev[rb], s));
      b->resorts += (int64_t)b->due.size();
    }
    if (ev1) HG_CUDA_TRY(cudaEventRecord(ev1, s));
    // per-scene argument tables [update args of S scenes | fused args of S
    // scenes]; an entry changes when its scene re-sorts (buffer swap), is
    // re-uploaded or changes dt, and the table is copied only then
    for (int i = 0; i < S; ++i) {
      hg_mpm *m = b->members[i];
      const hg_batch::Sig sg{m, m->cur, m->n, b->dts[i]};
      if (b->dirty || !(sg == b->sigs[i])) {
        b->sigs[i] = sg;
        cache[i] = make_args(m, b->dts[i], true);
        cache[S + i] = make_args(m, b->dts[i], false);
        b->dirty = true;
      }
    }
    if (b->dirty) {
      const int tb = b->tb;
      b->tb = (b->tb + 1) % hg_batch::NBUF;
      const auto w0 = std::chrono::steady_clock::now();
      HG_CUDA_TRY(cudaEventSynchronize(b->table_ev[tb]));
      b->wait_ms +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
      const size_t bytes = 2 * (size_t)S * sizeof(MixedArgs);
      std::memcpy(b->h_table[tb], cache, bytes);
      // ordered after the previous step's kernels, which read the table
      HG_CUDA_TRY(cudaMemcpyAsync(b->table.p, b->h_table[tb], bytes, cudaMemcpyHostToDevice, s));
      HG_CUDA_TRY(cudaEventRecord(b->table_ev[tb], s));
      b->dirty = false;
    }
    if (ev2) HG_CUDA_TRY(cudaEventRecord(ev2, s));
    return HG_OK;
  };
  int k = 0;
  // whole chunks replay a captured graph; event timing needs the per-step path
  while (!b->profile && nsteps - k >= CHUNK_STEPS) {
    hg_status st = prepare(nullptr, nullptr);
    if (st == HG_OK) st = batch_chunk_graph(b, S);
    if (st != HG_OK) return st;
    HG_CUDA_TRY(cudaGraphLaunch(b->chunk_exec, s));
    g_launches.fetch_add(b->chunk_launches, std::memory_order_relaxed);
    HG_CUDA_TRY(cudaEventRecord(b->out_ev, s));
    b->out_members = b->members;
    b->out_pending = true;
    for (hg_mpm *m : b->members) m->steps_since_rebin += CHUNK_STEPS;
    b->member_steps += (int64_t)S * CHUNK_STEPS;
    b->steps += CHUNK_STEPS;
    k += CHUNK_STEPS;
  }
  for (; k < nsteps; ++k) {
    cudaEvent_t ev[hg_batch::PROF_PHASES + 1] = {};
    if (b->profile) {
      while (b->prof_events.size() < b->prof_used + hg_batch::PROF_PHASES + 1) {
        cudaEvent_t e;
        HG_CUDA_TRY(cudaEventCreate(&e));
        b->prof_events.push_back(e);
      }
      for (int j = 0; j <= hg_batch::PROF_PHASES; ++j) ev[j] = b->prof_events[b->prof_used + j];
      b->prof_used += hg_batch::PROF_PHASES + 1;
      HG_CUDA_TRY(cudaEventRecord(ev[0], s));
    }
    hg_status st = prepare(ev[1], ev[2]);
    if (st != HG_OK) return st;
    const MixedArgs *dt = reinterpret_cast<const MixedArgs *>(b->table.p);
    const MixedArgs *db = dt + S;
    const int nsm = b->ctx->num_sms;
    HG_LAUNCH(kb_grid_update, nsm * update_per_sm(b->shape), THREADS, 0, s, dt, S,
              b->queue.p + 2);
    HG_CHECK_LAUNCH();
    if (b->profile) HG_CUDA_TRY(cudaEventRecord(ev[3], s));
    HG_LAUNCH(kb_g2p2g, nsm * fused_per_sm(b->shape), THREADS, 0, s, db, S, b->queue.p);
    HG_CHECK_LAUNCH();
    if (b->profile) HG_CUDA_TRY(cudaEventRecord(ev[4], s));
    for (hg_mpm *m : b->members) m->steps_since_rebin++;
    b->member_steps += S;
    b->steps++;
    if (!b->out_pending) {
      HG_LAUNCH(kb_gather_outside, (S + 127) / 128, 128, 0, s, db, S, b->outside.p);
      HG_CHECK_LAUNCH();
      HG_CUDA_TRY(cudaMemcpyAsync(b->h_outside, b->outside.p, 2 * sizeof(uint32_t) * S,
                                  cudaMemcpyDeviceToHost, s));
      HG_CUDA_TRY(cudaEventRecord(b->out_ev, s));
      b->out_members = b->members;
      b->out_pending = true;
    }
  }
  return HG_OK;
}

// ---- autotuning -------------------------------------------------------------

namespace {

// Picks, per kernel, the candidate with the least mean time per step.
void pick(hg_tune_report &r) {
  int bf = 0, bu = 0;
  for (int i = 1; i < r.candidates; ++i) {
    if (r.fused_ms[i] < r.fused_ms[bf]) bf = i;
    if (r.update_ms[i] < r.update_ms[bu]) bu = i;
  }
  r.chosen = hg_launch_shape{r.tried[bf].fused_ctas_per_sm, r.tried[bu].update_ctas_per_sm};
}

} // namespace

hg_status mixed_autotune(hg_mpm *m, double dt, int steps, hg_tune_report *report) {
  hg_tune_report r{};
  r.candidates = HG_TUNE_CANDIDATES;
  const bool prof0 = m->profile;
  hg_status st = HG_OK;
  if (!m->primed) st = prime(m);
  for (int i = 0; i < HG_TUNE_CANDIDATES && st == HG_OK; ++i) {
    r.tried[i] = TUNE_CANDIDATES[i];
    m->shape = TUNE_CANDIDATES[i];
    // one untimed step with the shape, then steps timed per kernel
    m->profile = false;
    st = mixed_step(m, dt, 1);
    if (st != HG_OK) break;
    m->profile = true;
    m->prof_used = 0;
    st = mixed_step(m, dt, steps);
    double g2p2g = 0.0, update = 0.0;
    int64_t n = 0;
    if (st == HG_OK) st = mixed_profile_read(m, &g2p2g, &update, &n);
    r.fused_ms[i] = n > 0 ? g2p2g / n : std::numeric_limits<double>::infinity();
    r.update_ms[i] = n > 0 ? update / n : std::numeric_limits<double>::infinity();
  }
  m->profile = false;
  m->prof_used = 0;
  r.steps = (int64_t)HG_TUNE_CANDIDATES * (1 + steps);
  // The whole step for every pair of a fused and an update shape, replayed
  // as graphs like the production steps (where the two kernels overlap under
  // programmatic dependent launch, which per-kernel events do not see): one
  // chunk captures and warms the pair's graph, two chunks are timed.
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (st == HG_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    st = fail(HG_ERR_CUDA, "cudaEventCreate");
  int bi = 0, bj = 0;
  cudaStream_t s = m->ctx->stream;
  for (int i = 0; i < HG_TUNE_CANDIDATES && st == HG_OK; ++i)
    for (int j = 0; j < HG_TUNE_CANDIDATES && st == HG_OK; ++j) {
      m->shape = hg_launch_shape{TUNE_CANDIDATES[i].fused_ctas_per_sm,
                                 TUNE_CANDIDATES[j].update_ctas_per_sm};
      st = mixed_step(m, dt, CHUNK_STEPS);
      if (st != HG_OK) break;
      float ms = 0.0f;
      cudaError_t e = cudaEventRecord(e0, s);
      if (e == cudaSuccess) st = mixed_step(m, dt, 2 * CHUNK_STEPS);
      if (e == cudaSuccess && st == HG_OK) e = cudaEventRecord(e1, s);
      if (e == cudaSuccess && st == HG_OK) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess && st == HG_OK) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess && st == HG_OK) st = cuda_fail(e, "autotune timing");
      r.step_ms[i][j] = (double)ms / (2 * CHUNK_STEPS);
      r.steps += 3 * CHUNK_STEPS;
      if (r.step_ms[i][j] < r.step_ms[bi][bj]) {
        bi = i;
        bj = j;
      }
    }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  m->profile = prof0;
  if (st != HG_OK) {
    m->shape = hg_launch_shape{0, 0};
    return st;
  }
  r.chosen = hg_launch_shape{TUNE_CANDIDATES[bi].fused_ctas_per_sm,
                             TUNE_CANDIDATES[bj].update_ctas_per_sm};
  m->shape = r.chosen;
  m->shape_set = true;
  tune_store(mixed_key(m), r.chosen);
  if (report) *report = r;
  // the step graphs of both particle buffers for the chosen shape and this
  // dt, so that later steps replay them instead of capturing one on first
  // use (capture only records the launches: the buffer swap is undone)
  for (int k = 0; k < 2; ++k) {
    st = mixed_chunk_graph(m, dt);
    m->cur ^= 1;
    if (st != HG_OK) {
      if (k == 0) m->cur ^= 1;
      return st;
    }
  }
  return HG_OK;
}

hg_status batch_autotune(hg_batch *b, int steps, hg_tune_report *report) {
  hg_tune_report r{};
  r.candidates = HG_TUNE_CANDIDATES;
  const bool prof0 = b->profile;
  int64_t points = 0;
  for (hg_mpm *m : b->members) points += m->n;
  b->shape_set = true; // the candidates, not the table, during the timing
  hg_status st = HG_OK;
  for (int i = 0; i < HG_TUNE_CANDIDATES && st == HG_OK; ++i) {
    r.tried[i] = TUNE_CANDIDATES[i];
    b->shape = TUNE_CANDIDATES[i];
    b->profile = false;
    st = batch_step(b, 1);
    if (st != HG_OK) break;
    b->profile = true;
    b->prof_used = 0;
    st = batch_step(b, steps);
    double ms[hg_batch::PROF_PHASES] = {0.0};
    int64_t n = 0;
    if (st == HG_OK) st = batch_profile_read(b, ms, &n);
    r.update_ms[i] = n > 0 ? ms[2] / n : std::numeric_limits<double>::infinity();
    r.fused_ms[i] = n > 0 ? ms[3] / n : std::numeric_limits<double>::infinity();
  }
  b->profile = prof0;
  b->prof_used = 0;
  if (st != HG_OK) {
    b->shape = hg_launch_shape{0, 0};
    b->shape_set = false;
    b->shape_class = -1;
    return st;
  }
  r.steps = (int64_t)HG_TUNE_CANDIDATES * (1 + steps);
  pick(r);
  b->shape = r.chosen;
  b->shape_class = batch_key(b, points)[3];
  tune_store(batch_key(b, points), r.chosen);
  // later steps follow the table again as the member mix changes
  b->shape_set = false;
  if (report) *report = r;
  return HG_OK;
}

hg_status tune_save(const char *path) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(HG_ERR_INVALID_ARGUMENT, "cannot open the tuning file for writing");
  for (const auto &e : g_tune)
    std::fprintf(f, "%lld %lld %lld %lld %d %d\n", (long long)e.first[0], (long long)e.first[1],
                 (long long)e.first[2], (long long)e.first[3], e.second.fused_ctas_per_sm,
                 e.second.update_ctas_per_sm);
  const bool ok = std::fclose(f) == 0;
  return ok ? HG_OK : fail(HG_ERR_INVALID_ARGUMENT, "writing the tuning file failed");
}

hg_status tune_load(const char *path) {
  FILE *f = std::fopen(path, "r");
  if (!f) return fail(HG_ERR_INVALID_ARGUMENT, "cannot open the tuning file");
  std::map<TuneKey, hg_launch_shape> add;
  long long k0, k1, k2, k3;
  int fu, up;
  int got;
  while ((got = std::fscanf(f, "%lld %lld %lld %lld %d %d", &k0, &k1, &k2, &k3, &fu, &up)) == 6) {
    if (fu < 0 || fu > 64 || up < 0 || up > 64) break;
    add[TuneKey{k0, k1, k2, k3}] = hg_launch_shape{fu, up};
  }
  const bool clean = got == EOF;
  std::fclose(f);
  if (!clean) return fail(HG_ERR_INVALID_ARGUMENT, "malformed tuning file");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (const auto &e : add) g_tune[e.first] = e.second;
  return HG_OK;
}

void tune_clear() {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.clear();
}

} // namespace hg
