// Penalty-DEM disk step (PenaltyImpactFrictionMap::flow / flowWithWeights,
// rigidbody2d/PenaltyImpactFrictionMap.cpp:1083-1149) in FP64.
//
// Compiled with --fmad=false: every record and force is evaluated with the
// operation order of the reference's Eigen expressions, and body forces are
// summed in the reference's order (gravity, plane contacts, circle-circle
// contacts in (first, second) order, kinematic contacts) by a per-body gather
// instead of atomics. The step is therefore deterministic and matches a serial
// FP64 evaluation of the reference bit for bit.
//
// Kernels per step:
//   kd_bodies_home / kd_fill broadphase: hash-grid counting sort of the disks
//                            by the cell of their AABB minimum. The cell width
//                            is 2 r_max (1 + 1e-6), so the partners of a disk
//                            lie in 3x3 cells; the result is the reference's
//                            candidate set {i < j : AABBs overlap}
//                            (SpatialGrid.cpp:14-19, 90-118), independent of
//                            the reference's own cell width.
//   kd_pairs_count / _emit   narrow phase (RigidBody2DSim.cpp:270-336 with
//                            q0 == q1, CollisionDetectionUtilities.cpp:3-101)
//                            and body-plane tests (RigidBody2DSim.cpp:777-842);
//                            count (keeping short partner lists), then emit
//                            sorted per-body contact lists. Candidates are
//                            filtered in FP32 on cell-relative offsets before
//                            the exact FP64 tests: FP64 runs at 1/64 of the
//                            FP32 rate on this part, and the filter leaves
//                            about one FP64 test per contact.
//   kd_contacts              collision-cache update with tangential-spring
//                            carry (PenaltyImpactFrictionMap.cpp:296-599) and
//                            the penalty force with Coulomb projection
//                            (616-1081, secondRootOfQuadratic 601-614).
//   kd_in_count / kd_in_fill incoming circle-circle contact lists per body.
//   kd_integrate             force gather, fixed-body zeroing and symplectic
//                            Euler (PenaltyImpactFrictionMap.cpp:1101-1114).
#include "hg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

namespace hg {

namespace {

constexpr int MAXP = 32; // partner list capacity per body and step
enum { K_PLANE = 0, K_CC = 1, K_KIN = 2 };
constexpr int RW = HG_DEM_RECORD_WIDTH;

struct D2 {
  double x, y;
};
__device__ __forceinline__ D2 dadd(D2 a, D2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ D2 dsub(D2 a, D2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ D2 dscl(double s, D2 a) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ double ddot(D2 a, D2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ double dsq(D2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double dnorm(D2 a) { return sqrt(dsq(a)); }
__device__ __forceinline__ D2 dnormalized(D2 a) {
  const double n2 = dsq(a);
  if (n2 > 0.0) {
    const double n = sqrt(n2);
    return {a.x / n, a.y / n};
  }
  return a;
}
__device__ __forceinline__ double dcross(D2 a, D2 b) { return a.x * b.y - a.y * b.x; }
// isfinite on the bit pattern (integer pipe; FP64 compares are scarce here)
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7FF) != 0x7FF;
}

__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, uint32_t mask) {
  return ((uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u) & mask;
}

__device__ __forceinline__ int64_t ckey(int kind, int a, int b) {
  return ((int64_t)kind << 60) | ((int64_t)a << 30) | (int64_t)b;
}

struct BroadArgs {
  int64_t n;
  double H; // cell width
  uint32_t mask;
  const double *mn; // 2 per box (min x, min y)
  const double *mx;
};

__global__ void kd_home(BroadArgs B, int2 *home, int32_t *bucket_count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= B.n) return;
  const int cx = (int)floor(B.mn[2 * i] / B.H), cy = (int)floor(B.mn[2 * i + 1] / B.H);
  home[i] = make_int2(cx, cy);
  atomicAdd(&bucket_count[cell_hash(cx, cy, B.mask)], 1);
}

__global__ void kd_fill(BroadArgs B, const int2 *__restrict__ home,
                        const int32_t *__restrict__ bucket_start, int32_t *cursor,
                        int32_t *items) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= B.n) return;
  const int2 c = home[i];
  const uint32_t b = cell_hash(c.x, c.y, B.mask);
  items[bucket_start[b] + atomicAdd(&cursor[b], 1)] = (int32_t)i;
}

// AABB::overlaps (SpatialGrid.cpp:14-19), inclusive on every side.
__device__ __forceinline__ bool box_overlap(const BroadArgs &B, int64_t i, int64_t j) {
  return (B.mx[2 * i] >= B.mn[2 * j] && B.mx[2 * i + 1] >= B.mn[2 * j + 1]) &&
         (B.mx[2 * j] >= B.mn[2 * i] && B.mx[2 * j + 1] >= B.mn[2 * i + 1]);
}

__device__ __forceinline__ void sort_small(int *keys, int n) {
  for (int i = 1; i < n; ++i) {
    const int k = keys[i];
    int j = i - 1;
    while (j >= 0 && keys[j] > k) {
      keys[j + 1] = keys[j];
      --j;
    }
    keys[j + 1] = k;
  }
}

// Per body, for the pair search: the home cell (the cell of the AABB
// minimum) and, in FP32, the offset of the centre from the home cell's
// corner and the radius, with the fixed flag and the active static planes
// (StaticPlaneCircleConstraint::isActive, StaticPlaneCircleConstraint.cpp:
// 12-17, in FP64) as bits. The FP64 arithmetic per body is a few operations;
// per candidate pair the search needs FP32 only, except for the exact tests
// of the pairs that survive the FP32 filter. Active static drums take the
// bits after the planes'. The home cell only has to be a
// consistent binning (the search covers the neighbouring cells), so it is
// floor(x_min / H) computed as x_min * (1 / H).
struct HomeArgs {
  int64_t n;
  double H, invH;
  uint32_t mask;
  int nplanes;
  double px[HG_MAX_PLANES][2], pn[HG_MAX_PLANES][2];
  int ndrums;
  double dx[HG_MAX_DRUMS][2], dr[HG_MAX_DRUMS];
  const double *q, *r;
  const uint8_t *fixed;
  float4 *rec; // 2 per body: (offset x, offset y, radius, flags), (home cell x, y)
  int32_t *bucket_count;
  // this step's per-body counters, zeroed here in place of memsets: contact
  // counts (3n + 1), pair fill (n), incoming counts (n + 1) and cursors (n)
  int32_t *per_body, *pfill, *in_count, *in_cursor;
};

enum : uint32_t { REL_FIXED = 1u, REL_PLANE0 = 2u };
static_assert(1 + HG_MAX_PLANES + HG_MAX_DRUMS <= 32, "static-object bits of the body record");

__global__ void kd_bodies_home(HomeArgs A) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  A.per_body[3 * i] = A.per_body[3 * i + 1] = A.per_body[3 * i + 2] = 0;
  A.pfill[i] = 0;
  A.in_count[i] = 0;
  A.in_cursor[i] = 0;
  if (i == 0) {
    A.per_body[3 * A.n] = 0;
    A.in_count[A.n] = 0;
  }
  // CircleGeometry::computeCollisionAABB (CircleGeometry.cpp:22-30), q0 == q1
  const double x = A.q[3 * i], y = A.q[3 * i + 1], ri = A.r[i];
  const int cx = (int)floor((x - ri) * A.invH), cy = (int)floor((y - ri) * A.invH);
  uint32_t flags = A.fixed[i] ? REL_FIXED : 0u;
  for (int k = 0; k < A.nplanes; ++k) {
    const double d = A.pn[k][0] * (x - A.px[k][0]) + A.pn[k][1] * (y - A.px[k][1]);
    if (d <= ri) flags |= REL_PLANE0 << k;
  }
  // StaticDrumCircleConstraint::isActive (StaticDrumCircleConstraint.cpp:7-13):
  // |x_drum - x|^2 >= (r_drum - r)^2; drum k is static object nplanes + k
  for (int k = 0; k < A.ndrums; ++k) {
    const double ex = A.dx[k][0] - x, ey = A.dx[k][1] - y, g = A.dr[k] - ri;
    if (ex * ex + ey * ey >= g * g) flags |= REL_PLANE0 << (A.nplanes + k);
  }
  // one 32-byte record: the FP32 part, then the home cell
  A.rec[2 * i] = make_float4((float)(x - (double)cx * A.H), (float)(y - (double)cy * A.H),
                             (float)ri, __uint_as_float(flags));
  A.rec[2 * i + 1] = make_float4(__int_as_float(cx), __int_as_float(cy), 0.0f, 0.0f);
  atomicAdd(&A.bucket_count[cell_hash(cx, cy, A.mask)], 1);
}

// Places each body in its bucket. bucket_pos holds the bucket starts and
// ends up holding the bucket ends (start + count).
__global__ void kd_fill_ends(int64_t n, uint32_t mask, const float4 *__restrict__ rec,
                             int32_t *bucket_pos, int32_t *items, uint32_t *status) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 h = rec[2 * i + 1];
  const int p = atomicAdd(&bucket_pos[cell_hash(__float_as_int(h.x), __float_as_int(h.y), mask)], 1);
  if (!HG_INDEX_OK(p, n, status)) return;
  items[p] = (int32_t)i;
}

// The per-body terms of kd_integrate that change only with the masses, the
// weights or the time step, with kd_integrate's operations: the gravity
// force 0 + M g (NearEarthGravityForce::computeForce) and dt / M, dt / Mi
// written as dt * (1 / M) (M = m0 w, Mi = I0 w:
// RigidBody2DState::updateCurrentMassUsingMassWeights).
__global__ void kd_body_terms(int64_t n, double dt, double gx, double gy,
                              const double *__restrict__ m0, const double *__restrict__ I0,
                              const double *__restrict__ w, double4 *terms) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double M = m0[j] * w[j], Mi = I0[j] * w[j];
  terms[j] = make_double4(0.0 + M * gx, 0.0 + M * gy, dt * (1.0 / M), dt * (1.0 / Mi));
}

constexpr int PW = 8; // partners per body kept by the counting pass

struct PairArgs {
  int64_t n;
  uint32_t mask;
  const float4 *rec; // body records of kd_bodies_home
  float Hf;  // cell width in FP32
  float tol; // FP32 filter slack
  const int32_t *bucket_end;
  const int32_t *bucket_count;
  const int32_t *items;
  const double *q;
  const double *r;
  int nstatic;        // static objects: the planes, then the drums
  int32_t *cnt;       // 3N counts [kind][body]
  uint32_t *plist;    // PW partners per body (fixed partners flagged by bit 31)
  int32_t *pfill;     // partners credited to each body (counting pass)
  const int32_t *off; // 3N+1 offsets (emit pass)
  int64_t *keys;      // emit pass output
  int64_t ccap;
  const int32_t *overflow; // emit pass: set when the contacts do not fit
  uint32_t *status;
};

// The contact test of a candidate pair (a, b), b's home cell offset by
// (dx, dy) from a's. The FP32 offsets from the home cells' corners give the
// centre distance to within about 1e-6 of a cell; the slack tol is 1e-4 of
// a cell. So a pair whose FP32 distance exceeds ra + rb + tol is no contact,
// and one whose FP32 distance is below ra + rb - tol is a contact under the
// reference's FP64 tests as well (its AABBs overlap and c0 < 0 by about
// 2 tol (ra + rb), far beyond FP64 rounding). Only the pairs in between take
// those tests: AABB overlap (SpatialGrid.cpp:14-19, with the AABB corners
// x -+ r evaluated as CircleGeometry.cpp:22-30 does) and
// ballBallCCDCollisionHappens with q0 == q1 (active iff c0 <= 0).
__device__ __forceinline__ bool is_contact(const PairArgs &A, float4 pa, float4 pb, int dx,
                                           int dy, int a, int b) {
  const float ex = (float)dx * A.Hf + (pb.x - pa.x);
  const float ey = (float)dy * A.Hf + (pb.y - pa.y);
  const float d2 = ex * ex + ey * ey;
  const float outer = pa.z + pb.z + A.tol, inner = pa.z + pb.z - A.tol;
  if (d2 > outer * outer) return false;
  if (inner > 0.0f && d2 < inner * inner) return true;
  const double xa = A.q[3 * a], ya = A.q[3 * a + 1], ra = A.r[a];
  const double xb = A.q[3 * b], yb = A.q[3 * b + 1], rb = A.r[b];
  if (!((xa + ra >= xb - rb && ya + ra >= yb - rb) && (xb + rb >= xa - ra && yb + rb >= ya - ra)))
    return false;
  const double ddx = xa - xb, ddy = ya - yb;
  const double c0 = (ddx * ddx + ddy * ddy) - (ra + rb) * (ra + rb);
  return c0 <= 0.0;
}

// Contact enumeration for body a as the first index: circle-circle with
// b > a non-fixed, kinematic with b fixed (any index; the reference swaps the
// fixed body into the second slot). Fixed bodies emit none.
//
// A partner b overlapping a's AABB has its home cell within one cell of a's
// (the cell width is at least every AABB's width), so the 3x3 cells around
// a's home cell hold every candidate.
template <class F>
__device__ __forceinline__ void for_each_partner(const PairArgs &A, int a, F &&found) {
  const float4 pa = A.rec[2 * a], ca = A.rec[2 * a + 1];
  const int2 ha = make_int2(__float_as_int(ca.x), __float_as_int(ca.y));
  // the nine bucket ranges first: independent loads instead of a chain
  int bs[9], be[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    const uint32_t bk = cell_hash(ha.x + c % 3 - 1, ha.y + c / 3 - 1, A.mask);
    be[c] = A.bucket_end[bk];
    bs[c] = be[c] - A.bucket_count[bk];
  }
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    const int dx = c % 3 - 1, dy = c / 3 - 1;
    const int cx = ha.x + dx, cy = ha.y + dy;
    for (int k = bs[c]; k < be[c]; ++k) {
      if (!HG_INDEX_OK(k, A.n, A.status)) break;
      const int b = A.items[k];
      if (!HG_INDEX_OK(b, A.n, A.status)) continue;
      if (b == a) continue;
      const float4 pb = A.rec[2 * b], cb = A.rec[2 * b + 1];
      if (__float_as_int(cb.x) != cx || __float_as_int(cb.y) != cy)
        continue; // bucket shared by another cell
      const bool bf = (__float_as_uint(pb.w) & REL_FIXED) != 0u;
      if (!(b > a || bf)) continue;
      if (!is_contact(A, pa, pb, dx, dy, a, b)) continue;
      found(b, bf);
    }
  }
}

// Counting pass over half of each neighbourhood: the home cell and the four
// cells after it in (dy, dx) order. A pair of bodies in different cells is
// met from exactly one of them (the offset from one home cell to the other is
// in the half, its negative is not); a pair within one cell is met from both
// and kept from the lower index. Each contact is credited to its first body
// (the lower index of two free bodies, the free body of a free-fixed pair,
// none for two fixed bodies) with atomics: per-kind counts, capped at MAXP,
// and the first PW partners in plist (in no particular order; the emission
// pass sorts them). The survivors of the FP32 filter take the same FP64 tests
// as the full search, which are symmetric in the two bodies.

__device__ __forceinline__ void credit(const PairArgs &A, int first, int second, bool kin,
                                       bool &overflow) {
  if (!HG_INDEX_OK(first, A.n, A.status)) return;
  int32_t *c = A.cnt + (kin ? 2 : 1) * A.n + first;
  if (atomicAdd(c, 1) >= MAXP) {
    atomicSub(c, 1);
    overflow = true;
    return;
  }
  const int slot = atomicAdd(A.pfill + first, 1);
  if (slot < PW) A.plist[(int64_t)first * PW + slot] = (uint32_t)second | (kin ? 0x80000000u : 0u);
}

// cell c of the half neighbourhood: (0, 0), (1, 0), (-1, 1), (0, 1), (1, 1)
__device__ __forceinline__ int half_dx(int c) { return c == 0 ? 0 : (c == 1 ? 1 : c - 3); }
__device__ __forceinline__ int half_dy(int c) { return c >= 2 ? 1 : 0; }

// One thread per body over its five cells: fewer loads of the body's own
// record than kd_pairs_count when the bodies alone fill the GPU.
__global__ void kd_pairs_count_body(PairArgs A) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t n = A.n;
  const int a = (int)(blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (a >= n) return;
  const float4 pa = A.rec[2 * a], ca = A.rec[2 * a + 1];
  const uint32_t flags = __float_as_uint(pa.w);
  const bool af = (flags & REL_FIXED) != 0u;
  if (!af) A.cnt[a] = __popc(flags >> 1); // static planes
  const int2 ha = make_int2(__float_as_int(ca.x), __float_as_int(ca.y));
  int bs[5], be[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const uint32_t bk = cell_hash(ha.x + half_dx(c), ha.y + half_dy(c), A.mask);
    be[c] = A.bucket_end[bk];
    bs[c] = be[c] - A.bucket_count[bk];
  }
  bool overflow = false;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const int dx = half_dx(c), dy = half_dy(c);
    const int cx = ha.x + dx, cy = ha.y + dy;
    for (int k = bs[c]; k < be[c]; ++k) {
      if (!HG_INDEX_OK(k, n, A.status)) break;
      const int b = A.items[k];
      if (!HG_INDEX_OK(b, n, A.status)) continue;
      if (b == a || (c == 0 && b < a)) continue;
      const float4 pb = A.rec[2 * b], cb = A.rec[2 * b + 1];
      if (__float_as_int(cb.x) != cx || __float_as_int(cb.y) != cy)
        continue; // bucket shared by another cell
      const bool bf = (__float_as_uint(pb.w) & REL_FIXED) != 0u;
      if (af && bf) continue;
      if (!is_contact(A, pa, pb, dx, dy, a, b)) continue;
      if (af) credit(A, b, a, true, overflow);
      else if (bf) credit(A, a, b, true, overflow);
      else credit(A, min(a, b), max(a, b), false, overflow);
    }
  }
  if (overflow) atomicOr(A.status, (uint32_t)HG_STATUS_CELL_OVERFLOW);
}

// One thread per (body, cell of the half neighbourhood): thread t takes cell
// t / n of body t % n, so a warp's lanes read consecutive bodies' records and
// each thread follows one bucket instead of five.
__global__ void kd_pairs_count(PairArgs A) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t n = A.n;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 5 * n) return;
  const int c = (int)(t / n);
  const int a = (int)(t - (int64_t)c * n);
  const float4 pa = A.rec[2 * a], ca = A.rec[2 * a + 1];
  const uint32_t flags = __float_as_uint(pa.w);
  const bool af = (flags & REL_FIXED) != 0u;
  if (c == 0 && !af) A.cnt[a] = __popc(flags >> 1); // static planes
  const int dx = half_dx(c), dy = half_dy(c);
  const int cx = __float_as_int(ca.x) + dx, cy = __float_as_int(ca.y) + dy;
  const uint32_t bk = cell_hash(cx, cy, A.mask);
  const int be = A.bucket_end[bk], bs = be - A.bucket_count[bk];
  if (bs >= be) return;
  bool overflow = false;
  for (int k = bs; k < be; ++k) {
    if (!HG_INDEX_OK(k, n, A.status)) break;
    const int b = A.items[k];
    if (!HG_INDEX_OK(b, n, A.status)) continue;
    if (b == a || (c == 0 && b < a)) continue;
    const float4 pb = A.rec[2 * b], cb = A.rec[2 * b + 1];
    if (__float_as_int(cb.x) != cx || __float_as_int(cb.y) != cy)
      continue; // bucket shared by another cell
    const bool bf = (__float_as_uint(pb.w) & REL_FIXED) != 0u;
    if (af && bf) continue;
    if (!is_contact(A, pa, pb, dx, dy, a, b)) continue;
    if (af) credit(A, b, a, true, overflow);
    else if (bf) credit(A, a, b, true, overflow);
    else credit(A, min(a, b), max(a, b), false, overflow);
  }
  if (overflow) atomicOr(A.status, (uint32_t)HG_STATUS_CELL_OVERFLOW);
}

// Emission pass: sorted per-body contact keys at the scanned offsets. Lists
// of at most PW partners come from the counting pass; longer ones are
// searched again (the same partners, the first MAXP of each kind).
__global__ void kd_pairs_emit(PairArgs A) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t n = A.n;
  const int a = (int)(blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (a >= n) return;
  const int npl = A.cnt[a], ncc = A.cnt[n + a], nkin = A.cnt[2 * n + a];
  if (npl + ncc + nkin == 0 || *A.overflow) return;
  const int64_t o0 = A.off[a], o1 = A.off[n + a], o2 = A.off[2 * n + a];
  if (o0 + npl > A.ccap || o1 + ncc > A.ccap || o2 + nkin > A.ccap) {
    atomicOr(A.status, (uint32_t)HG_STATUS_CONTACT_OVERFLOW);
    return;
  }
  const uint32_t flags = __float_as_uint(A.rec[2 * a].w);
  int j = 0;
  for (int k = 0; k < A.nstatic; ++k)
    if (flags & (REL_PLANE0 << k)) A.keys[o0 + j++] = ckey(K_PLANE, a, k);
  if (ncc + nkin <= PW) {
    // odd-even transposition sort of the flagged indices: circle-circle
    // partners ascending, then the fixed ones ascending
    uint32_t L[PW];
    const uint32_t *lst = A.plist + (int64_t)a * PW;
#pragma unroll
    for (int k = 0; k < PW; ++k) L[k] = k < ncc + nkin ? lst[k] : 0xFFFFFFFFu;
#pragma unroll
    for (int p = 0; p < PW; ++p)
#pragma unroll
      for (int i = p & 1; i + 1 < PW; i += 2) {
        const uint32_t lo = min(L[i], L[i + 1]), hi = max(L[i], L[i + 1]);
        L[i] = lo;
        L[i + 1] = hi;
      }
#pragma unroll
    for (int k = 0; k < PW; ++k) {
      if (k < ncc) A.keys[o1 + k] = ckey(K_CC, a, (int)L[k]);
      else if (k < ncc + nkin) A.keys[o2 + (k - ncc)] = ckey(K_KIN, a, (int)(L[k] & 0x7FFFFFFFu));
    }
    return;
  }
  int cc[MAXP], kin[MAXP];
  int mc = 0, mk = 0;
  for_each_partner(A, a, [&](int b, bool bf) {
    if (bf) {
      if (mk < MAXP) kin[mk++] = b;
    } else if (mc < MAXP) {
      cc[mc++] = b;
    }
  });
  sort_small(cc, mc);
  sort_small(kin, mk);
  for (int k = 0; k < mc; ++k) A.keys[o1 + k] = ckey(K_CC, a, cc[k]);
  for (int k = 0; k < mk; ++k) A.keys[o2 + k] = ckey(K_KIN, a, kin[k]);
}

// Capacity guard between the counting and the emission pass: when the total
// exceeds the contact capacity the step keeps no contacts (and reports
// HG_STATUS_CONTACT_OVERFLOW) instead of writing past the buffers.
__global__ void kd_check_capacity(int64_t n, const int32_t *__restrict__ off, int64_t ccap,
                                  int32_t *overflow, uint32_t *status) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const bool over = (int64_t)off[3 * n] > ccap;
    *overflow = over ? 1 : 0;
    if (over) atomicOr(status, (uint32_t)HG_STATUS_CONTACT_OVERFLOW);
  }
}

__global__ void kd_drop_if_overflow(int64_t n, const int32_t *__restrict__ overflow,
                                    int32_t *cnt, int32_t *off) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  if (!*overflow) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= 3 * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    cnt[i] = 0;
    off[i] = 0;
  }
}

struct ContactArgs {
  int64_t n;
  double dt;
  int weighted;
  double kn, kt, gn, gt, mu;
  int nplanes;
  double px[HG_MAX_PLANES][2], pn[HG_MAX_PLANES][2];
  int ndrums; // static objects nplanes .. nplanes + ndrums - 1
  double dx[HG_MAX_DRUMS][2], dr[HG_MAX_DRUMS];
  const double *q, *v, *r, *w;
  const int32_t *count; // device count (total contacts)
  const int64_t *keys;
  double *rec;
  const int64_t *old_keys;
  const double *old_rec;
  const int32_t *old_count; // device count of the previous step's contacts
  int64_t ccap;
  uint32_t *status;
};

__device__ __forceinline__ int find_old(const ContactArgs &C, int64_t key) {
  int lo = 0, hi = min((int64_t)*C.old_count, C.ccap) - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int64_t k = C.old_keys[mid];
    if (k == key) return mid;
    if (k < key) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// secondRootOfQuadratic (PenaltyImpactFrictionMap.cpp:601-614)
__device__ __forceinline__ double second_root(double a, double b, double c, double ds) {
  if (b > 0.0) return (2.0 * c) / (-b - ds);
  return (-b + ds) / (2.0 * a);
}

__global__ void kd_contacts(ContactArgs C) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t total = min((int64_t)*C.count, C.ccap);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t key = C.keys[k];
    const int kind = (int)(key >> 60);
    const int a = (int)((key >> 30) & 0x3FFFFFFF);
    const int b = (int)(key & 0x3FFFFFFF);
    if (!HG_INDEX_OK(a, C.n, C.status) ||
        !HG_INDEX_OK(b, kind == K_PLANE ? (int64_t)(C.nplanes + C.ndrums) : C.n, C.status))
      continue;
    const D2 qa{C.q[3 * a], C.q[3 * a + 1]};
    const D2 va{C.v[3 * a], C.v[3 * a + 1]};
    const double wa = C.v[3 * a + 2];
    double depth, weight;
    D2 n, cp{0.0, 0.0}, r0, r1{0.0, 0.0}, vrel;
    const double ra = C.r[a];
    if (kind == K_PLANE && b >= C.nplanes) { // PenaltyImpactFrictionMap.cpp:361-401
      // StaticDrumCircleConstraint.cpp:100-159: the normal points from the
      // disk's centre to the drum's; the contact point is the disk's point
      // farthest from the drum's centre
      const int dk = b - C.nplanes;
      const D2 xd{C.dx[dk][0], C.dx[dk][1]};
      n = dnormalized(dsub(xd, qa));
      cp = dsub(qa, dscl(ra, n));
      weight = C.weighted ? C.w[a] : 1.0;
      const double gap = -(dnorm(dsub(xd, qa)) - (C.dr[dk] - ra));
      depth = gap < 0.0 ? gap : 0.0; // std::min(0.0, gap)
      r0 = dscl(-ra, n);
      const D2 t0{-r0.y, r0.x};
      const D2 arm = dsub(cp, xd);
      const D2 tp{-arm.y, arm.x};
      const D2 vp{0.0 + 0.0 * tp.x, 0.0 + 0.0 * tp.y}; // the drum is static
      vrel = dsub(dadd(va, dscl(wa, t0)), vp);
    } else if (kind == K_PLANE) { // PenaltyImpactFrictionMap.cpp:316-359
      const D2 xp{C.px[b][0], C.px[b][1]};
      n = D2{C.pn[b][0], C.pn[b][1]};
      cp = dsub(qa, dscl(ra, n));
      weight = C.weighted ? C.w[a] : 1.0;
      depth = fmin(0.0, ddot(n, dsub(qa, xp)) - ra);
      r0 = dscl(-ra, n);
      const D2 t0{-r0.y, r0.x};
      const D2 arm = dsub(cp, xp);
      const D2 tp{-arm.y, arm.x};
      const D2 vp{0.0 + 0.0 * tp.x, 0.0 + 0.0 * tp.y};
      vrel = dsub(dadd(va, dscl(wa, t0)), vp);
    } else {
      const D2 qb{C.q[3 * b], C.q[3 * b + 1]};
      const double rb = C.r[b];
      n = dnormalized(dsub(qa, qb));
      depth = fmin(0.0, dnorm(dsub(qa, qb)) - ra - rb);
      const D2 vb{C.v[3 * b], C.v[3 * b + 1]};
      const double wb = C.v[3 * b + 2];
      if (kind == K_CC) { // CircleCircleConstraint.cpp:171-233
        cp = dadd(qa, dscl(ra / (ra + rb), dsub(qb, qa)));
        weight = C.weighted ? (C.w[a] + C.w[b]) * 0.5 : 1.0;
        r0 = dsub(cp, qa);
        r1 = dsub(cp, qb);
        const D2 t0{-r0.y, r0.x}, t1{-r1.y, r1.x};
        vrel = dsub(dsub(dadd(va, dscl(wa, t0)), vb), dscl(wb, t1));
      } else { // KinematicObjectCircleConstraint.cpp
        cp = dsub(qa, dscl(ra, n));
        weight = C.weighted ? C.w[a] : 1.0;
        r0 = dscl(-ra, n);
        const D2 t{-r0.y, r0.x};
        const D2 arm = dsub(cp, qb);
        const D2 tk{-arm.y, arm.x};
        const D2 vk = dadd(vb, dscl(wb, tk));
        vrel = dsub(dadd(va, dscl(wa, t)), vk);
      }
    }
    // tangential spring carry
    D2 ds;
    const int o = find_old(C, key);
    if (o >= 0) {
      ds = D2{C.old_rec[(int64_t)o * RW + 6], C.old_rec[(int64_t)o * RW + 7]};
      ds = dadd(ds, dscl(C.dt, vrel));
    } else {
      ds = dscl(C.dt, vrel);
    }
    ds = dsub(ds, dscl(ddot(n, ds), n));
    // penalty force (PenaltyImpactFrictionMap.cpp:616-1081)
    const double w = weight;
    const D2 vt = dsub(vrel, dscl(ddot(n, vrel), n));
    const D2 vn = dsub(vrel, vt);
    const D2 fn = dsub(dscl(-C.kn * w * depth, n), dscl(0.5 * C.gn * w, vn));
    D2 ft = dsub(dscl(-C.kt * w, ds), dscl(0.5 * C.gt * w, vt));
    const double mu_fn = C.mu * dnorm(fn);
    const double ftn = dnorm(ft);
    if (0.5 * C.gt * w * dnorm(vt) > mu_fn) {
      ds = D2{0.0, 0.0};
      ft = dscl(-0.5 * C.gt * w, vt);
      ft = dnormalized(ft);
      ft = dscl(mu_fn, ft);
    } else if (ftn > mu_fn) {
      const double qa_ = C.kt * w * C.kt * w * dsq(ds);
      const double qb_ = C.kt * w * C.gt * w * ddot(ds, vt);
      const double qc_ = 0.25 * C.gt * w * C.gt * w * ddot(vt, vt) - C.mu * C.mu * dsq(fn);
      const double dscr = qb_ * qb_ - 4 * qa_ * qc_;
      const double root1 = second_root(qa_, qb_, qc_, sqrt(dscr));
      const D2 nds = dscl(root1, ds);
      ft = dsub(dscl(-C.kt * w, nds), dscl(0.5 * C.gt * w, vt));
      ds = nds;
    }
    double *o_ = C.rec + k * RW;
    o_[0] = kind;
    o_[1] = a;
    o_[2] = b;
    o_[3] = depth;
    o_[4] = n.x;
    o_[5] = n.y;
    o_[6] = ds.x;
    o_[7] = ds.y;
    o_[8] = vrel.x;
    o_[9] = vrel.y;
    o_[10] = r0.x;
    o_[11] = r0.y;
    o_[12] = r1.x;
    o_[13] = r1.y;
    o_[14] = weight;
    o_[15] = cp.x;
    o_[16] = cp.y;
    o_[17] = fn.x;
    o_[18] = fn.y;
    o_[19] = ft.x;
    o_[20] = ft.y;
    o_[21] = 0.0;
  }
}

__global__ void kd_in_count(int64_t n, const int32_t *__restrict__ off,
                            const int64_t *__restrict__ keys, int32_t *in_count) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  // circle-circle contacts occupy [off[n], off[2n])
  const int s = off[n], e = off[2 * n];
  for (int64_t k = s + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < e;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&in_count[keys[k] & 0x3FFFFFFF], 1);
}

__global__ void kd_in_fill(int64_t n, const int32_t *__restrict__ off,
                           const int64_t *__restrict__ keys,
                           const int32_t *__restrict__ in_off, int32_t *in_cursor,
                           int32_t *in_list) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int s = off[n], e = off[2 * n];
  for (int64_t k = s + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < e;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(keys[k] & 0x3FFFFFFF);
    in_list[in_off[b] + atomicAdd(&in_cursor[b], 1)] = (int32_t)k;
  }
}

__global__ void kd_integrate(int64_t n, double dt, double *q, double *v,
                             const double4 *__restrict__ terms,
                             const uint8_t *__restrict__ fixed,
                             const int32_t *__restrict__ cnt, const int32_t *__restrict__ off,
                             const double *__restrict__ rec, const int32_t *__restrict__ in_count,
                             const int32_t *__restrict__ in_off, int32_t *in_list,
                             uint32_t *status) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  // gravity and dt / M, dt / Mi from kd_body_terms
  const double4 bt = terms[j];
  double Fx = bt.x, Fy = bt.y, T = 0.0;
  auto total = [&](int64_t k, D2 &f) {
    const double *r = rec + k * RW;
    f = dadd(D2{r[17], r[18]}, D2{r[19], r[20]});
  };
  // circle vs plane
  for (int64_t k = off[j], e = off[j] + cnt[j]; k < e; ++k) {
    D2 f;
    total(k, f);
    Fx += f.x;
    Fy += f.y;
    T += dcross(D2{rec[k * RW + 10], rec[k * RW + 11]}, f);
  }
  // circle vs circle: contributions as the second body come from first
  // indices below j, i.e. before j's own list in the reference's loop.
  {
    int *lst = in_list + in_off[j];
    const int c = in_count[j];
    for (int i = 1; i < c; ++i) { // contact indices sorted = first indices sorted
      const int key = lst[i];
      int t = i - 1;
      while (t >= 0 && lst[t] > key) {
        lst[t + 1] = lst[t];
        --t;
      }
      lst[t + 1] = key;
    }
    for (int i = 0; i < c; ++i) {
      const int64_t k = lst[i];
      if (!HG_INDEX_OK(k, off[3 * n], status)) continue;
      D2 f;
      total(k, f);
      Fx -= f.x;
      Fy -= f.y;
      T -= dcross(D2{rec[k * RW + 12], rec[k * RW + 13]}, f);
    }
  }
  for (int64_t k = off[n + j], e = off[n + j] + cnt[n + j]; k < e; ++k) {
    D2 f;
    total(k, f);
    Fx += f.x;
    Fy += f.y;
    T += dcross(D2{rec[k * RW + 10], rec[k * RW + 11]}, f);
  }
  // kinematic circle vs circle
  for (int64_t k = off[2 * n + j], e = off[2 * n + j] + cnt[2 * n + j]; k < e; ++k) {
    D2 f;
    total(k, f);
    Fx += f.x;
    Fy += f.y;
    T += dcross(D2{rec[k * RW + 10], rec[k * RW + 11]}, f);
  }
  if (fixed[j]) Fx = Fy = T = 0.0;
  // v1 = v0 + dt Minv F ; q1 = q0 + dt v1
  const double v0 = v[3 * j] + bt.z * Fx;
  const double v1 = v[3 * j + 1] + bt.z * Fy;
  const double v2 = v[3 * j + 2] + bt.w * T;
  v[3 * j] = v0;
  v[3 * j + 1] = v1;
  v[3 * j + 2] = v2;
  const double q0 = q[3 * j] + dt * v0, q1 = q[3 * j + 1] + dt * v1, q2 = q[3 * j + 2] + dt * v2;
  q[3 * j] = q0;
  q[3 * j + 1] = q1;
  q[3 * j + 2] = q2;
  if (!finite_bits(q0) || !finite_bits(q1) || !finite_bits(v0) || !finite_bits(v1))
    atomicOr(status, (uint32_t)HG_STATUS_NONFINITE);
}

// ---- mixed precision: the same contact law and integration with FP32
// arithmetic; positions, the pairwise position difference, the contact point
// and the position update stay FP64 (a millimetre overlap taken from
// metre-scale coordinates in FP32 would be lost to cancellation). Records and
// velocities keep the FP64 storage of the FP64 path, holding FP32 values, so
// the broadphase, history relabelling, collision-cache export, coupling and
// checkpoints are shared.
struct F2 {
  float x, y;
};
__device__ __forceinline__ F2 fadd(F2 a, F2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ F2 fsub(F2 a, F2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ F2 fscl(float s, F2 a) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ float fdot(F2 a, F2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float fnrm(F2 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ F2 fnormalized(F2 a) {
  const float n2 = fdot(a, a);
  if (n2 > 0.0f) {
    const float n = sqrtf(n2);
    return {a.x / n, a.y / n};
  }
  return a;
}
__device__ __forceinline__ float fcross(F2 a, F2 b) { return a.x * b.y - a.y * b.x; }

__global__ void kdx_contacts(ContactArgs C) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t total = min((int64_t)*C.count, C.ccap);
  const float dt = (float)C.dt, kn = (float)C.kn, kt = (float)C.kt, gn = (float)C.gn,
              gt = (float)C.gt, mu = (float)C.mu;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t key = C.keys[k];
    const int kind = (int)(key >> 60);
    const int a = (int)((key >> 30) & 0x3FFFFFFF);
    const int b = (int)(key & 0x3FFFFFFF);
    if (!HG_INDEX_OK(a, C.n, C.status) ||
        !HG_INDEX_OK(b, kind == K_PLANE ? (int64_t)(C.nplanes + C.ndrums) : C.n, C.status))
      continue;
    const double qax = C.q[3 * a], qay = C.q[3 * a + 1];
    const F2 va{(float)C.v[3 * a], (float)C.v[3 * a + 1]};
    const float wa = (float)C.v[3 * a + 2];
    const float ra = (float)C.r[a];
    float depth, weight;
    F2 n, r0, r1{0.0f, 0.0f}, vrel;
    double cpx, cpy;
    if (kind == K_PLANE && b >= C.nplanes) { // PenaltyImpactFrictionMap.cpp:361-401
      const int dk = b - C.nplanes;
      const double ex = C.dx[dk][0] - qax, ey = C.dx[dk][1] - qay; // FP64 difference
      const F2 e{(float)ex, (float)ey};
      n = fnormalized(e); // towards the drum's centre
      // -(|e| - (R - r)) as ((R - r)^2 - |e|^2) / (|e| + R - r): the
      // cancelling difference in FP64, the rest in FP32
      const double g = C.dr[dk] - C.r[a];
      const double g2 = g * g - (ex * ex + ey * ey);
      depth = g2 < 0.0 ? (float)g2 / (fnrm(e) + (float)g) : 0.0f;
      weight = C.weighted ? (float)C.w[a] : 1.0f;
      r0 = fscl(-ra, n);
      cpx = qax + (double)r0.x;
      cpy = qay + (double)r0.y;
      vrel = fadd(va, fscl(wa, F2{-r0.y, r0.x})); // the drum is static
    } else if (kind == K_PLANE) { // PenaltyImpactFrictionMap.cpp:316-359
      n = F2{(float)C.pn[b][0], (float)C.pn[b][1]};
      // penetration from FP64 positions (a difference of nearly equal terms)
      const double dist = C.pn[b][0] * (qax - C.px[b][0]) + C.pn[b][1] * (qay - C.px[b][1]);
      depth = (float)fmin(0.0, dist - C.r[a]);
      weight = C.weighted ? (float)C.w[a] : 1.0f;
      r0 = fscl(-ra, n);
      cpx = qax + (double)r0.x;
      cpy = qay + (double)r0.y;
      vrel = fadd(va, fscl(wa, F2{-r0.y, r0.x})); // the plane is static
    } else {
      const double qbx = C.q[3 * b], qby = C.q[3 * b + 1];
      const float rb = (float)C.r[b];
      const double dx = qax - qbx, dy = qay - qby; // FP64 difference
      const F2 d{(float)dx, (float)dy};
      n = fnormalized(d);
      // |d| - (ra + rb) as (|d|^2 - (ra + rb)^2) / (|d| + ra + rb): the
      // cancelling difference in FP64, the rest in FP32
      const double rs = C.r[a] + C.r[b];
      const double g2 = (dx * dx + dy * dy) - rs * rs;
      depth = g2 < 0.0 ? (float)g2 / (fnrm(d) + (float)rs) : 0.0f;
      const F2 vb{(float)C.v[3 * b], (float)C.v[3 * b + 1]};
      const float wb = (float)C.v[3 * b + 2];
      if (kind == K_CC) { // CircleCircleConstraint.cpp:171-233
        weight = C.weighted ? (float)((C.w[a] + C.w[b]) * 0.5) : 1.0f;
        r0 = fscl(-(ra / (ra + rb)), d); // p - xa = ra/(ra+rb) (xb - xa)
        r1 = fadd(d, r0);                // p - xb
        vrel = fsub(fsub(fadd(va, fscl(wa, F2{-r0.y, r0.x})), vb), fscl(wb, F2{-r1.y, r1.x}));
      } else { // KinematicObjectCircleConstraint.cpp
        weight = C.weighted ? (float)C.w[a] : 1.0f;
        r0 = fscl(-ra, n);
        const F2 arm = fadd(d, r0); // p - xb
        const F2 vk = fadd(vb, fscl(wb, F2{-arm.y, arm.x}));
        vrel = fsub(fadd(va, fscl(wa, F2{-r0.y, r0.x})), vk);
      }
      cpx = qax + (double)r0.x;
      cpy = qay + (double)r0.y;
    }
    // tangential spring carry
    F2 ds;
    const int o = find_old(C, key);
    if (o >= 0) {
      ds = F2{(float)C.old_rec[(int64_t)o * RW + 6], (float)C.old_rec[(int64_t)o * RW + 7]};
      ds = fadd(ds, fscl(dt, vrel));
    } else {
      ds = fscl(dt, vrel);
    }
    ds = fsub(ds, fscl(fdot(n, ds), n));
    // penalty force (PenaltyImpactFrictionMap.cpp:616-1081)
    const float w = weight;
    const F2 vt = fsub(vrel, fscl(fdot(n, vrel), n));
    const F2 vn = fsub(vrel, vt);
    const F2 fn = fsub(fscl(-kn * w * depth, n), fscl(0.5f * gn * w, vn));
    F2 ft = fsub(fscl(-kt * w, ds), fscl(0.5f * gt * w, vt));
    const float mu_fn = mu * fnrm(fn);
    if (0.5f * gt * w * fnrm(vt) > mu_fn) {
      ds = F2{0.0f, 0.0f};
      ft = fscl(mu_fn, fnormalized(fscl(-0.5f * gt * w, vt)));
    } else if (fnrm(ft) > mu_fn) {
      // secondRootOfQuadratic (PenaltyImpactFrictionMap.cpp:601-614)
      const float qa_ = kt * w * kt * w * fdot(ds, ds);
      const float qb_ = kt * w * gt * w * fdot(ds, vt);
      const float qc_ = 0.25f * gt * w * gt * w * fdot(vt, vt) - mu * mu * fdot(fn, fn);
      const float sq = sqrtf(fmaxf(qb_ * qb_ - 4.0f * qa_ * qc_, 0.0f));
      const float root1 = qb_ > 0.0f ? (2.0f * qc_) / (-qb_ - sq) : (-qb_ + sq) / (2.0f * qa_);
      ds = fscl(root1, ds);
      ft = fsub(fscl(-kt * w, ds), fscl(0.5f * gt * w, vt));
    }
    double *o_ = C.rec + k * RW;
    o_[0] = kind;
    o_[1] = a;
    o_[2] = b;
    o_[3] = depth;
    o_[4] = n.x;
    o_[5] = n.y;
    o_[6] = ds.x;
    o_[7] = ds.y;
    o_[8] = vrel.x;
    o_[9] = vrel.y;
    o_[10] = r0.x;
    o_[11] = r0.y;
    o_[12] = r1.x;
    o_[13] = r1.y;
    o_[14] = weight;
    o_[15] = cpx;
    o_[16] = cpy;
    o_[17] = fn.x;
    o_[18] = fn.y;
    o_[19] = ft.x;
    o_[20] = ft.y;
    o_[21] = 0.0;
  }
}

// Force gather (the FP64 kernel's summation order) and symplectic Euler in
// FP32; q += dt v in FP64.
__global__ void kdx_integrate(int64_t n, double dt, double *q, double *v,
                              const double4 *__restrict__ terms,
                              const uint8_t *__restrict__ fixed,
                              const int32_t *__restrict__ cnt, const int32_t *__restrict__ off,
                              const double *__restrict__ rec,
                              const int32_t *__restrict__ in_count,
                              const int32_t *__restrict__ in_off, int32_t *in_list,
                              uint32_t *status) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double4 bt = terms[j];
  float Fx = (float)bt.x, Fy = (float)bt.y, T = 0.0f;
  auto add = [&](int64_t k, int which, float sign) {
    const double *r = rec + k * RW;
    const F2 f = fadd(F2{(float)r[17], (float)r[18]}, F2{(float)r[19], (float)r[20]});
    Fx += sign * f.x;
    Fy += sign * f.y;
    T += sign * fcross(F2{(float)r[10 + 2 * which], (float)r[11 + 2 * which]}, f);
  };
  for (int64_t k = off[j], e = off[j] + cnt[j]; k < e; ++k) add(k, 0, 1.0f);
  {
    int *lst = in_list + in_off[j];
    const int c = in_count[j];
    for (int i = 1; i < c; ++i) { // contact indices sorted = first indices sorted
      const int key = lst[i];
      int t = i - 1;
      while (t >= 0 && lst[t] > key) {
        lst[t + 1] = lst[t];
        --t;
      }
      lst[t + 1] = key;
    }
    for (int i = 0; i < c; ++i)
      if (HG_INDEX_OK(lst[i], off[3 * n], status)) add(lst[i], 1, -1.0f);
  }
  for (int64_t k = off[n + j], e = off[n + j] + cnt[n + j]; k < e; ++k) add(k, 0, 1.0f);
  for (int64_t k = off[2 * n + j], e = off[2 * n + j] + cnt[2 * n + j]; k < e; ++k)
    add(k, 0, 1.0f);
  if (fixed[j]) Fx = Fy = T = 0.0f;
  const float v0 = (float)v[3 * j] + (float)bt.z * Fx;
  const float v1 = (float)v[3 * j + 1] + (float)bt.z * Fy;
  const float v2 = (float)v[3 * j + 2] + (float)bt.w * T;
  v[3 * j] = v0;
  v[3 * j + 1] = v1;
  v[3 * j + 2] = v2;
  const double q0 = q[3 * j] + dt * (double)v0, q1 = q[3 * j + 1] + dt * (double)v1,
               q2 = q[3 * j + 2] + dt * (double)v2;
  q[3 * j] = q0;
  q[3 * j + 1] = q1;
  q[3 * j + 2] = q2;
  if (!finite_bits(q0) || !finite_bits(q1) || !isfinite(v0) || !isfinite(v1))
    atomicOr(status, (uint32_t)HG_STATUS_NONFINITE);
}


// Candidate pairs of explicit boxes (SpatialGrid::getPotentialOverlaps).
template <bool EMIT>
__global__ void kd_box_pairs(BroadArgs B, const int2 *__restrict__ home,
                             const int32_t *__restrict__ bstart,
                             const int32_t *__restrict__ bcount,
                             const int32_t *__restrict__ items, int32_t *cnt,
                             const int32_t *__restrict__ off, int32_t *pairs, int64_t cap,
                             uint32_t *status) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= B.n) return;
  int list[MAXP];
  int np = 0;
  bool overflow = false;
  const int cx0 = (int)floor(B.mn[2 * a] / B.H) - 1, cy0 = (int)floor(B.mn[2 * a + 1] / B.H) - 1;
  const int cx1 = (int)floor(B.mx[2 * a] / B.H), cy1 = (int)floor(B.mx[2 * a + 1] / B.H);
  for (int cy = cy0; cy <= cy1; ++cy)
    for (int cx = cx0; cx <= cx1; ++cx) {
      const uint32_t bk = cell_hash(cx, cy, B.mask);
      for (int k = bstart[bk], e = bstart[bk] + bcount[bk]; k < e; ++k) {
        const int b = items[k];
        if (b <= a) continue;
        const int2 hb = home[b];
        if (hb.x != cx || hb.y != cy) continue;
        if (!box_overlap(B, a, b)) continue;
        if (np < MAXP) list[np++] = b;
        else overflow = true;
      }
    }
  if (overflow) atomicOr(status, (uint32_t)HG_STATUS_CELL_OVERFLOW);
  if (!EMIT) {
    cnt[a] = np;
    return;
  }
  sort_small(list, np);
  const int64_t o = off[a];
  for (int k = 0; k < np; ++k)
    if (o + k < cap) {
      pairs[2 * (o + k)] = (int32_t)a;
      pairs[2 * (o + k) + 1] = list[k];
    }
}

inline int blocks_for(int64_t n, int t) { return (int)std::max<int64_t>(1, (n + t - 1) / t); }


uint32_t table_bits(int64_t n) {
  uint32_t bits = 4;
  while (((int64_t)1 << bits) < 2 * n && bits < 30) ++bits;
  return bits;
}

// Broadphase tables for n boxes: bucket counts/starts, items and home cells.
hg_status build_buckets(cudaStream_t s, BroadArgs &B, int32_t *bcount, int32_t *bstart,
                        int32_t *cursor, int32_t *items, int2 *home, int32_t *scan_tmp) {
  const int64_t T = (int64_t)B.mask + 1;
  HG_CUDA_TRY(cudaMemsetAsync(bcount, 0, sizeof(int32_t) * T, s));
  HG_CUDA_TRY(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * T, s));
  if (B.n == 0) return HG_OK;
  HG_LAUNCH(kd_home, blocks_for(B.n, 256), 256, 0, s, B, home, bcount);
  HG_CHECK_LAUNCH();
  hg_status st = exclusive_scan_i32(bcount, bstart, T, scan_tmp, s);
  if (st != HG_OK) return st;
  HG_LAUNCH(kd_fill, blocks_for(B.n, 256), 256, 0, s, B, home, bstart, cursor, items);
  HG_CHECK_LAUNCH();
  return HG_OK;
}


} // namespace

hg_status dem_alloc(hg_dem *d) {
  const int64_t N = std::max<int64_t>(d->cap, 1);
  const int64_t C = std::max<int64_t>(d->ccap, 1);
  const uint32_t bits = table_bits(N);
  d->mask = (1u << bits) - 1u;
  const int64_t T = (int64_t)d->mask + 1;
  int64_t tmp = std::max(scan_tmp_size(3 * N + 1), scan_tmp_size(T));
  tmp = std::max(tmp, scan_tmp_size(N + 1));
  hg_status st;
  if ((st = d->status.alloc(1)) || (st = d->q.alloc(3 * N)) || (st = d->v.alloc(3 * N)) ||
      (st = d->r.alloc(N)) || (st = d->m0.alloc(N)) || (st = d->I0.alloc(N)) ||
      (st = d->w.alloc(N)) || (st = d->minv.alloc(4 * N)) || (st = d->fixed.alloc(N)) ||
      (st = d->brec.alloc(2 * N)) || (st = d->pfill.alloc(N)) || (st = d->plist.alloc(PW * N)) ||
      (st = d->bcount.alloc(T)) || (st = d->bstart.alloc(T)) ||
      (st = d->items.alloc(N)) || (st = d->scan_tmp.alloc(tmp)) ||
      (st = d->c_count.alloc(2)) || (st = d->per_body.alloc(3 * N + 1)) ||
      (st = d->per_body_off.alloc(3 * N + 1)) || (st = d->ckey[0].alloc(C)) ||
      (st = d->ckey[1].alloc(C)) || (st = d->crec[0].alloc(C * RW)) ||
      (st = d->crec[1].alloc(C * RW)) || (st = d->in_count.alloc(N + 1)) ||
      (st = d->in_off.alloc(N + 1)) || (st = d->in_list.alloc(C)) ||
      (st = d->in_cursor.alloc(N)) || (st = d->overflow.alloc(1)))
    return st;
  cudaStream_t s = dem_stream(d);
  HG_CUDA_TRY(cudaMemsetAsync(d->status.p, 0, sizeof(uint32_t), s));
  HG_CUDA_TRY(cudaMemsetAsync(d->c_count.p, 0, 2 * sizeof(int32_t), s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status dem_reset_history(hg_dem *d) {
  HG_CUDA_TRY(cudaMemsetAsync(d->c_count.p, 0, 2 * sizeof(int32_t), dem_stream(d)));
  d->history_valid = false;
  return HG_OK;
}

hg_status dem_prepare(hg_dem *d, double dt) {
  if ((d->inv_valid && d->terms_dt == dt) || d->n == 0) return HG_OK;
  HG_LAUNCH(kd_body_terms, blocks_for(d->n, 256), 256, 0, dem_stream(d), d->n, dt, d->p.g[0],
            d->p.g[1], d->m0.p, d->I0.p, d->w.p, reinterpret_cast<double4 *>(d->minv.p));
  HG_CHECK_LAUNCH();
  d->inv_valid = true;
  d->terms_dt = dt;
  return HG_OK;
}

// The contact law's grid: one resident wave (the SM count times the blocks
// of 256 threads that fit on an SM at once: 3 for the FP64 law's registers,
// 4 for the mixed one's), so that the grid-stride loop runs no partial
// second wave.
void dem_set_launch_shapes(hg_dem *d) {
  int per_sm = 0;
  cudaError_t e = d->p.precision == HG_PRECISION_MIXED
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kdx_contacts, 256, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kd_contacts, 256, 0);
  if (e != cudaSuccess || per_sm < 1) {
    (void)cudaGetLastError();
    per_sm = 3;
  }
  d->contact_grid = d->ctx->num_sms * per_sm;
}

hg_status dem_step(hg_dem *d, double dt, int weighted) {
  cudaStream_t s = dem_stream(d);
  const int64_t n = d->n;
  if (n == 0) return HG_OK;
  hg_status st;
  if ((st = dem_prepare(d, dt))) return st;
  // the hash table grows with the live body count (at most the capacity's)
  const uint32_t mask = (1u << table_bits(n)) - 1u;
  {
    // hash-grid counting sort of the bodies by home cell
    const int64_t T = (int64_t)mask + 1;
    HG_CUDA_TRY(cudaMemsetAsync(d->bcount.p, 0, sizeof(int32_t) * T, s));
    HomeArgs H;
    H.n = n;
    H.H = d->cell_h;
    H.invH = 1.0 / d->cell_h;
    H.mask = mask;
    H.nplanes = d->p.nplanes;
    H.ndrums = d->p.ndrums;
    for (int k = 0; k < HG_MAX_DRUMS; ++k) {
      H.dx[k][0] = d->p.dx[k][0];
      H.dx[k][1] = d->p.dx[k][1];
      H.dr[k] = d->p.dr[k];
    }
    for (int k = 0; k < HG_MAX_PLANES; ++k)
      for (int c = 0; c < 2; ++c) {
        H.px[k][c] = d->p.px[k][c];
        H.pn[k][c] = d->p.pn[k][c];
      }
    H.q = d->q.p;
    H.r = d->r.p;
    H.fixed = d->fixed.p;
    H.rec = d->brec.p;
    H.bucket_count = d->bcount.p;
    H.per_body = d->per_body.p;
    H.pfill = d->pfill.p;
    H.in_count = d->in_count.p;
    H.in_cursor = d->in_cursor.p;
    HG_LAUNCH_PDL(kd_bodies_home, blocks_for(n, 256), 256, 0, s, H);
    HG_CHECK_LAUNCH();
    if ((st = exclusive_scan_i32(d->bcount.p, d->bstart.p, T, d->scan_tmp.p, s))) return st;
    HG_LAUNCH_PDL(kd_fill_ends, blocks_for(n, 256), 256, 0, s, n, mask, d->brec.p, d->bstart.p,
              d->items.p, d->status.p);
    HG_CHECK_LAUNCH();
  }
  PairArgs A;
  A.n = n;
  A.mask = mask;
  A.rec = d->brec.p;
  A.Hf = (float)d->cell_h;
  A.tol = (float)(1.0e-4 * d->cell_h);
  A.plist = d->plist.p;
  A.bucket_end = d->bstart.p;
  A.bucket_count = d->bcount.p;
  A.items = d->items.p;
  A.q = d->q.p;
  A.r = d->r.p;
  A.nstatic = d->p.nplanes + d->p.ndrums;
  A.cnt = d->per_body.p;
  A.off = d->per_body_off.p;
  const int nb = 1 - d->cc; // buffer receiving this step's contacts
  A.keys = d->ckey[nb].p;
  A.ccap = d->ccap;
  A.overflow = d->overflow.p;
  A.status = d->status.p;
  A.pfill = d->pfill.p;
  // (per_body and pfill were zeroed by kd_bodies_home)
  // Below about one body per thread slot of the GPU, five threads per body
  // hide the bucket walks' latency; above it, one thread per body reads each
  // body's record once.
  if (n < (int64_t)d->ctx->num_sms * 1024)
    HG_LAUNCH_PDL(kd_pairs_count, blocks_for(5 * n, 128), 128, 0, s, A);
  else
    HG_LAUNCH_PDL(kd_pairs_count_body, blocks_for(n, 128), 128, 0, s, A);
  HG_CHECK_LAUNCH();
  // offsets, the contact-capacity check (all contacts dropped when the list
  // would overflow) and the contact count
  const bool small = 3 * n + 1 <= small_scan_max();
  if (small) {
    ScanLimit lim;
    lim.limit = d->ccap;
    lim.overflow = d->overflow.p;
    lim.status = d->status.p;
    lim.status_bit = HG_STATUS_CONTACT_OVERFLOW;
    lim.total = d->c_count.p + nb;
    if ((st = exclusive_scan_i32_limited(d->per_body.p, d->per_body_off.p, 3 * n + 1, lim, s)))
      return st;
  } else {
    if ((st = exclusive_scan_i32(d->per_body.p, d->per_body_off.p, 3 * n + 1, d->scan_tmp.p,
                                 s)))
      return st;
    HG_LAUNCH_PDL(kd_check_capacity, 1, 32, 0, s, n, d->per_body_off.p, d->ccap, d->overflow.p,
              d->status.p);
    HG_CHECK_LAUNCH();
    HG_LAUNCH_PDL(kd_drop_if_overflow, blocks_for(3 * n + 1, 256), 256, 0, s, n, d->overflow.p,
              d->per_body.p, d->per_body_off.p);
    HG_CHECK_LAUNCH();
  }
  HG_LAUNCH_PDL(kd_pairs_emit, blocks_for(n, 128), 128, 0, s, A);
  HG_CHECK_LAUNCH();
  if (!small)
    HG_CUDA_TRY(cudaMemcpyAsync(d->c_count.p + nb, d->per_body_off.p + 3 * n, sizeof(int32_t),
                                cudaMemcpyDeviceToDevice, s));
  ContactArgs Cg;
  Cg.n = n;
  Cg.dt = dt;
  Cg.weighted = weighted;
  Cg.kn = d->p.kn;
  Cg.kt = d->p.kt;
  Cg.gn = d->p.gn;
  Cg.gt = d->p.gt;
  Cg.mu = d->p.mu;
  Cg.nplanes = d->p.nplanes;
  Cg.ndrums = d->p.ndrums;
  for (int k = 0; k < HG_MAX_DRUMS; ++k) {
    Cg.dx[k][0] = d->p.dx[k][0];
    Cg.dx[k][1] = d->p.dx[k][1];
    Cg.dr[k] = d->p.dr[k];
  }
  for (int k = 0; k < HG_MAX_PLANES; ++k)
    for (int c = 0; c < 2; ++c) {
      Cg.px[k][c] = d->p.px[k][c];
      Cg.pn[k][c] = d->p.pn[k][c];
    }
  Cg.q = d->q.p;
  Cg.v = d->v.p;
  Cg.r = d->r.p;
  Cg.w = d->w.p;
  Cg.count = d->c_count.p + nb;
  Cg.keys = d->ckey[nb].p;
  Cg.rec = d->crec[nb].p;
  Cg.old_keys = d->ckey[d->cc].p;
  Cg.old_rec = d->crec[d->cc].p;
  Cg.old_count = d->c_count.p + d->cc;
  Cg.ccap = d->ccap;
  Cg.status = d->status.p;
  // The contact law is launched in stream order: scheduled while
  // kd_pairs_emit is still running, its one-wave grid-stride launch took
  // 10 us longer per step on 28,000 contacts (2.8 per disk); every other
  // launch of the step is programmatic.
  const int cgrid = d->contact_grid > 0 ? d->contact_grid : d->ctx->num_sms * 3;
  if (d->p.precision == HG_PRECISION_MIXED)
    HG_LAUNCH(kdx_contacts, cgrid, 256, 0, s, Cg);
  else
    HG_LAUNCH(kd_contacts, cgrid, 256, 0, s, Cg);
  HG_CHECK_LAUNCH();
  // (in_count and in_cursor were zeroed by kd_bodies_home)
  HG_LAUNCH_PDL(kd_in_count, d->ctx->num_sms * 2, 256, 0, s, n, d->per_body_off.p, d->ckey[nb].p,
            d->in_count.p);
  HG_CHECK_LAUNCH();
  if ((st = exclusive_scan_i32(d->in_count.p, d->in_off.p, n + 1, d->scan_tmp.p, s))) return st;
  HG_LAUNCH_PDL(kd_in_fill, d->ctx->num_sms * 2, 256, 0, s, n, d->per_body_off.p, d->ckey[nb].p,
            d->in_off.p, d->in_cursor.p, d->in_list.p);
  HG_CHECK_LAUNCH();
  auto integrate = d->p.precision == HG_PRECISION_MIXED ? kdx_integrate : kd_integrate;
  HG_LAUNCH_PDL(integrate, blocks_for(n, 128), 128, 0, s, n, dt, d->q.p, d->v.p,
            reinterpret_cast<const double4 *>(d->minv.p), d->fixed.p, d->per_body.p,
            d->per_body_off.p,
            d->crec[nb].p, d->in_count.p, d->in_off.p, d->in_list.p, d->status.p);
  HG_CHECK_LAUNCH();
  d->cc = nb;
  d->history_valid = true;
  return HG_OK;
}

// ---- contact history after bodies are removed -------------------------------
//
// PenaltyImpactFrictionMap::deleteCacheEntries / relabelEntries
// (PenaltyImpactFrictionMap.cpp:1199-1278): contacts of removed bodies are
// dropped and the others renumbered. The map is monotone, so the list stays
// sorted by (kind, first, second) and a stable compaction keeps it valid for
// the next step's history lookup.
namespace {

__device__ __forceinline__ bool relabel_one(int64_t key, const int32_t *map, int64_t nmap,
                                            int64_t &out, int32_t &a2, int32_t &b2) {
  const int64_t kind = key >> 60;
  const int64_t a = (key >> 30) & 0x3FFFFFFF, b = key & 0x3FFFFFFF;
  a2 = a < nmap ? map[a] : -1;
  b2 = kind == 0 ? (int32_t)b : (b < nmap ? map[b] : -1); // kind 0: plane index
  out = (kind << 60) | ((int64_t)a2 << 30) | (int64_t)b2;
  return a2 >= 0 && b2 >= 0;
}

__global__ void kd_relabel_keep(int64_t ccap, const int32_t *__restrict__ count,
                                const int64_t *__restrict__ keys, const int32_t *__restrict__ map,
                                int64_t nmap, int32_t *keep) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k > ccap) return;
  const int64_t c = min((int64_t)*count, ccap);
  int64_t nk;
  int32_t a2, b2;
  keep[k] = (k < c && relabel_one(keys[k], map, nmap, nk, a2, b2)) ? 1 : 0;
}

__global__ void kd_relabel_move(int64_t ccap, const int32_t *__restrict__ count,
                                const int64_t *__restrict__ keys, const double *__restrict__ rec,
                                const int32_t *__restrict__ map, int64_t nmap,
                                const int32_t *__restrict__ off, int64_t *okeys, double *orec,
                                int32_t *ocount) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = min((int64_t)*count, ccap);
  if (k == 0) *ocount = off[c];
  if (k >= c) return;
  int64_t nk;
  int32_t a2, b2;
  if (!relabel_one(keys[k], map, nmap, nk, a2, b2)) return;
  const int64_t o = off[k];
  okeys[o] = nk;
  for (int j = 0; j < RW; ++j) orec[o * RW + j] = rec[k * RW + j];
  orec[o * RW + 1] = (double)a2;
  orec[o * RW + 2] = (double)b2;
}

} // namespace

hg_status dem_relabel_device(hg_dem *d, const int32_t *map, int64_t nmap) {
  if (!d->history_valid) return HG_OK;
  cudaStream_t s = dem_stream(d);
  const int64_t C = d->ccap;
  DevBuf<int32_t> keep, off, tmp;
  hg_status st;
  if ((st = keep.alloc(C + 1)) || (st = off.alloc(C + 1)) || (st = tmp.alloc(scan_tmp_size(C + 1))))
    return st;
  const int nb = 1 - d->cc;
  HG_LAUNCH(kd_relabel_keep, blocks_for(C + 1, 256), 256, 0, s, C, d->c_count.p + d->cc,
            d->ckey[d->cc].p, map, nmap, keep.p);
  HG_CHECK_LAUNCH();
  if ((st = exclusive_scan_i32(keep.p, off.p, C + 1, tmp.p, s))) return st;
  HG_LAUNCH(kd_relabel_move, blocks_for(C + 1, 256), 256, 0, s, C, d->c_count.p + d->cc,
            d->ckey[d->cc].p, d->crec[d->cc].p, map, nmap, off.p, d->ckey[nb].p,
            d->crec[nb].p, d->c_count.p + nb);
  HG_CHECK_LAUNCH();
  d->cc = nb;
  return HG_OK;
}

hg_status dem_relabel(hg_dem *d, const int32_t *map_host, int64_t nmap) {
  if (!d->history_valid) return HG_OK;
  cudaStream_t s = dem_stream(d);
  DevBuf<int32_t> map;
  hg_status st;
  if ((st = map.alloc(std::max<int64_t>(nmap, 1)))) return st;
  if (nmap > 0)
    HG_CUDA_TRY(cudaMemcpyAsync(map.p, map_host, sizeof(int32_t) * nmap, cudaMemcpyHostToDevice, s));
  if ((st = dem_relabel_device(d, map.p, nmap))) return st;
  // the map was copied from the caller's memory: it may go once this returns
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

namespace {

// Moves kept bodies to their new slots (old_to_new, monotone) in scratch
// arrays; the caller copies the scratch back.
__global__ void kd_compact_bodies(int64_t n_old, const int32_t *__restrict__ map,
                                  const double *__restrict__ q, const double *__restrict__ v,
                                  const double *__restrict__ r, const double *__restrict__ m0,
                                  const double *__restrict__ I0, const double *__restrict__ w,
                                  const uint8_t *__restrict__ fixed, double *tq, double *tv,
                                  double *tr, double *tm, double *tI, double *tw, uint8_t *tf) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_old) return;
  const int32_t j = map[i];
  if (j < 0) return;
  for (int c = 0; c < 3; ++c) {
    tq[3 * (int64_t)j + c] = q[3 * i + c];
    tv[3 * (int64_t)j + c] = v[3 * i + c];
  }
  tr[j] = r[i];
  tm[j] = m0[i];
  tI[j] = I0[i];
  tw[j] = w[i];
  tf[j] = fixed[i];
}

__global__ void kd_ones(double *a, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = 1.0;
}

} // namespace

hg_status dem_edit(hg_dem *d, int64_t n_old, const int32_t *map_host, int64_t n_keep,
                   int64_t n_add, const double *q, const double *v, const double *r,
                   const double *m, const double *I, const uint8_t *fixed) {
  cudaStream_t s = dem_stream(d);
  hg_status st;
  DevBuf<int32_t> map;
  if (n_old > 0) {
    DevBuf<double> tq, tv, tr, tm, tI, tw;
    DevBuf<uint8_t> tf;
    const int64_t k = std::max<int64_t>(n_keep, 1);
    if ((st = map.alloc(n_old)) || (st = tq.alloc(3 * k)) || (st = tv.alloc(3 * k)) ||
        (st = tr.alloc(k)) || (st = tm.alloc(k)) || (st = tI.alloc(k)) || (st = tw.alloc(k)) ||
        (st = tf.alloc(k)))
      return st;
    HG_CUDA_TRY(cudaMemcpyAsync(map.p, map_host, sizeof(int32_t) * n_old, cudaMemcpyHostToDevice, s));
    HG_LAUNCH(kd_compact_bodies, blocks_for(n_old, 256), 256, 0, s, n_old, map.p, d->q.p, d->v.p,
              d->r.p, d->m0.p, d->I0.p, d->w.p, d->fixed.p, tq.p, tv.p, tr.p, tm.p, tI.p, tw.p,
              tf.p);
    HG_CHECK_LAUNCH();
    if (n_keep > 0) {
      HG_CUDA_TRY(cudaMemcpyAsync(d->q.p, tq.p, sizeof(double) * 3 * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->v.p, tv.p, sizeof(double) * 3 * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->r.p, tr.p, sizeof(double) * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->m0.p, tm.p, sizeof(double) * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->I0.p, tI.p, sizeof(double) * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->w.p, tw.p, sizeof(double) * n_keep, cudaMemcpyDeviceToDevice, s));
      HG_CUDA_TRY(cudaMemcpyAsync(d->fixed.p, tf.p, n_keep, cudaMemcpyDeviceToDevice, s));
    }
    if ((st = dem_relabel_device(d, map.p, n_old))) return st;
  }
  if (n_add > 0) {
    const int64_t o = n_keep;
    HG_CUDA_TRY(cudaMemcpyAsync(d->q.p + 3 * o, q, sizeof(double) * 3 * n_add, cudaMemcpyHostToDevice, s));
    HG_CUDA_TRY(cudaMemcpyAsync(d->v.p + 3 * o, v, sizeof(double) * 3 * n_add, cudaMemcpyHostToDevice, s));
    HG_CUDA_TRY(cudaMemcpyAsync(d->r.p + o, r, sizeof(double) * n_add, cudaMemcpyHostToDevice, s));
    HG_CUDA_TRY(cudaMemcpyAsync(d->m0.p + o, m, sizeof(double) * n_add, cudaMemcpyHostToDevice, s));
    HG_CUDA_TRY(cudaMemcpyAsync(d->I0.p + o, I, sizeof(double) * n_add, cudaMemcpyHostToDevice, s));
    if (fixed) {
      HG_CUDA_TRY(cudaMemcpyAsync(d->fixed.p + o, fixed, n_add, cudaMemcpyHostToDevice, s));
    } else {
      HG_CUDA_TRY(cudaMemsetAsync(d->fixed.p + o, 0, n_add, s));
    }
    HG_LAUNCH(kd_ones, blocks_for(n_add, 256), 256, 0, s, d->w.p + o, n_add);
    HG_CHECK_LAUNCH();
  }
  d->n = n_keep + n_add;
  d->inv_valid = false;
  return HG_OK;
}


hg_status dem_download_contacts(hg_dem *d, int64_t cap, double *rec, int64_t *count) {
  cudaStream_t s = dem_stream(d);
  int32_t c = 0;
  if (d->history_valid) {
    HG_CUDA_TRY(cudaMemcpyAsync(&c, d->c_count.p + d->cc, sizeof(int32_t),
                                cudaMemcpyDeviceToHost, s));
    HG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  const int64_t total = std::min<int64_t>(c, d->ccap);
  *count = total;
  const int64_t k = std::min<int64_t>(total, cap);
  if (k > 0) {
    HG_CUDA_TRY(cudaMemcpyAsync(rec, d->crec[d->cc].p, sizeof(double) * RW * k,
                                cudaMemcpyDeviceToHost, s));
    HG_CUDA_TRY(cudaStreamSynchronize(s));
    // drum contacts are static objects after the planes on the device; the
    // export names them by kind and drum index
    if (d->p.ndrums > 0)
      for (int64_t i = 0; i < k; ++i) {
        double *o = rec + i * RW;
        if (o[0] == (double)K_PLANE && o[2] >= (double)d->p.nplanes) {
          o[0] = (double)HG_DEM_KIND_DRUM;
          o[2] -= (double)d->p.nplanes;
        }
      }
  }
  return HG_OK;
}

hg_status dem_candidate_pairs(hg_context *ctx, int64_t n, const double *mn, const double *mx,
                              int64_t cap, int32_t *pairs, int64_t *count) {
  cudaStream_t s = ctx->stream;
  *count = 0;
  if (n == 0) return HG_OK;
  double H = 0.0, amax = 0.0;
  for (int64_t i = 0; i < 2 * n; ++i) {
    H = std::max(H, mx[i] - mn[i]);
    amax = std::max(amax, std::max(std::fabs(mn[i]), std::fabs(mx[i])));
  }
  H = H * (1.0 + 1.0e-6);
  if (amax / H > 1.0e9) return fail(HG_ERR_INVALID_ARGUMENT, "boxes too small for their coordinates");
  const uint32_t bits = table_bits(n);
  const int64_t T = (int64_t)1 << bits;
  DevBuf<double> dmn, dmx;
  DevBuf<int2> home;
  DevBuf<int32_t> bcount, bstart, bcursor, items, cnt, off, tmp, dpairs;
  DevBuf<uint32_t> status;
  hg_status st;
  if ((st = dmn.alloc(2 * n)) || (st = dmx.alloc(2 * n)) || (st = home.alloc(n)) ||
      (st = bcount.alloc(T)) || (st = bstart.alloc(T)) || (st = bcursor.alloc(T)) ||
      (st = items.alloc(n)) || (st = cnt.alloc(n + 1)) || (st = off.alloc(n + 1)) ||
      (st = tmp.alloc(std::max(scan_tmp_size(T), scan_tmp_size(n + 1)))) ||
      (st = status.alloc(1)))
    return st;
  HG_CUDA_TRY(cudaMemcpyAsync(dmn.p, mn, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s));
  HG_CUDA_TRY(cudaMemcpyAsync(dmx.p, mx, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s));
  HG_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(uint32_t), s));
  HG_CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (n + 1), s));
  BroadArgs B;
  B.n = n;
  B.H = H;
  B.mask = (uint32_t)(T - 1);
  B.mn = dmn.p;
  B.mx = dmx.p;
  if ((st = build_buckets(s, B, bcount.p, bstart.p, bcursor.p, items.p, home.p, tmp.p))) return st;
  HG_LAUNCH(kd_box_pairs<false>, blocks_for(n, 128), 128, 0, s, B, home.p, bstart.p, bcount.p,
            items.p, cnt.p, off.p, nullptr, 0, status.p);
  HG_CHECK_LAUNCH();
  if ((st = exclusive_scan_i32(cnt.p, off.p, n + 1, tmp.p, s))) return st;
  int32_t total = 0;
  uint32_t word = 0;
  HG_CUDA_TRY(cudaMemcpyAsync(&total, off.p + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaMemcpyAsync(&word, status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  if (word & HG_STATUS_CELL_OVERFLOW)
    return fail(HG_ERR_CAPACITY, "more than 32 overlapping boxes for one box");
  if ((st = dpairs.alloc(2 * (int64_t)std::max<int32_t>(total, 1)))) return st;
  HG_LAUNCH(kd_box_pairs<true>, blocks_for(n, 128), 128, 0, s, B, home.p, bstart.p, bcount.p,
            items.p, cnt.p, off.p, dpairs.p, (int64_t)total, status.p);
  HG_CHECK_LAUNCH();
  const int64_t k = std::min<int64_t>(total, cap);
  if (k > 0)
    HG_CUDA_TRY(cudaMemcpyAsync(pairs, dpairs.p, sizeof(int32_t) * 2 * k, cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  *count = total;
  return HG_OK;
}

} // namespace hg

// ---- allocation-free candidate-pair search -------------------------------------
//
// The same broadphase as hg_dem_candidate_pairs, with every device temporary
// placed in one file-scope __device__ array instead of cudaMalloc'd buffers.

namespace hg {
namespace {

constexpr int64_t SP_MAX_BOXES = HG_STATIC_PAIRS_MAX_BOXES;
constexpr int64_t SP_MAX_PAIRS = HG_STATIC_PAIRS_MAX_PAIRS;
constexpr uint32_t SP_TABLE_BITS = 15; // 32768 buckets >= 2 * SP_MAX_BOXES
constexpr int64_t SP_TABLE = (int64_t)1 << SP_TABLE_BITS;
static_assert(SP_TABLE >= 2 * SP_MAX_BOXES, "hash table too small");

constexpr size_t sp_align(size_t b) { return (b + 255) & ~(size_t)255; }
// Byte offsets of the regions inside the scratch array.
constexpr size_t SP_MN = 0;
constexpr size_t SP_MX = SP_MN + sp_align(sizeof(double) * 2 * SP_MAX_BOXES);
constexpr size_t SP_HOME = SP_MX + sp_align(sizeof(double) * 2 * SP_MAX_BOXES);
constexpr size_t SP_BCOUNT = SP_HOME + sp_align(sizeof(int2) * SP_MAX_BOXES);
constexpr size_t SP_BSTART = SP_BCOUNT + sp_align(sizeof(int32_t) * SP_TABLE);
constexpr size_t SP_BCURSOR = SP_BSTART + sp_align(sizeof(int32_t) * SP_TABLE);
constexpr size_t SP_ITEMS = SP_BCURSOR + sp_align(sizeof(int32_t) * SP_TABLE);
constexpr size_t SP_CNT = SP_ITEMS + sp_align(sizeof(int32_t) * SP_MAX_BOXES);
constexpr size_t SP_OFF = SP_CNT + sp_align(sizeof(int32_t) * (SP_MAX_BOXES + 1));
constexpr size_t SP_TMP = SP_OFF + sp_align(sizeof(int32_t) * (SP_MAX_BOXES + 1));
// the scans run over the bucket table and over the per-box counts
constexpr size_t SP_TMP_INTS = 256;
static_assert(SP_TMP_INTS >= (size_t)scan_tmp_size(SP_TABLE > SP_MAX_BOXES + 1 ? SP_TABLE
                                                                             : SP_MAX_BOXES + 1),
              "scan scratch region too small for the largest scan");
constexpr size_t SP_PAIRS = SP_TMP + sp_align(sizeof(int32_t) * SP_TMP_INTS);
constexpr size_t SP_STATUS = SP_PAIRS + sp_align(sizeof(int32_t) * 2 * SP_MAX_PAIRS);
constexpr size_t SP_BYTES = SP_STATUS + 256;

} // namespace
} // namespace hg

// Every GPU that loads the library holds this array (about 3.4 MB) until the
// process exits. Host code must not pass its name to a kernel: on the host
// the name is a stand-in, not a device address; the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_pairs_scratch[hg::SP_BYTES];

namespace hg {
namespace {

std::mutex g_sp_mutex;
unsigned char *g_sp_ptr[256] = {};

// Device address of g_pairs_scratch on the current device, looked up once per
// device (the lookup initialises the module on that device). The address is
// kept for the life of the process: a cudaDeviceReset of the device unloads
// the module and ends every context of this library on it, this address
// included, so no call may follow a reset.
hg_status static_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= 256) return fail(HG_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_sp_mutex);
  if (!g_sp_ptr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_pairs_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_pairs_scratch)");
    g_sp_ptr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_sp_ptr[device];
  return HG_OK;
}

} // namespace
} // namespace hg

extern "C" hg_status hg_dem_candidate_pairs_static(hg_context *ctx, int64_t n,
                                                   const double *aabb_min,
                                                   const double *aabb_max, int64_t cap,
                                                   int32_t *pairs, int64_t *count) {
  using namespace hg;
  if (!ctx || !count || n < 0 || (n > 0 && (!aabb_min || !aabb_max)) || (cap > 0 && !pairs) ||
      cap < 0)
    return fail(HG_ERR_INVALID_ARGUMENT, "bad argument");
  if (n > SP_MAX_BOXES)
    return fail(HG_ERR_CAPACITY, "hg_dem_candidate_pairs_static takes at most " +
                                     std::to_string(SP_MAX_BOXES) + " boxes, got " +
                                     std::to_string(n));
  *count = 0;
  double H = 0.0, amax = 0.0;
  for (int64_t i = 0; i < 2 * n; ++i) {
    if (!std::isfinite(aabb_min[i]) || !std::isfinite(aabb_max[i]) || !(aabb_min[i] < aabb_max[i]))
      return fail(HG_ERR_INVALID_ARGUMENT, "boxes must be finite with min < max");
    H = std::max(H, aabb_max[i] - aabb_min[i]);
    amax = std::max(amax, std::max(std::fabs(aabb_min[i]), std::fabs(aabb_max[i])));
  }
  if (n == 0) return HG_OK;
  H = H * (1.0 + 1.0e-6);
  if (amax / H > 1.0e9) return fail(HG_ERR_INVALID_ARGUMENT, "boxes too small for their coordinates");
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != ctx->device) cudaSetDevice(ctx->device);
  struct Restore {
    int dev;
    ~Restore() {
      if (dev >= 0) cudaSetDevice(dev);
    }
  } restore{prev != ctx->device ? prev : -1};
  unsigned char *base = nullptr;
  hg_status st = static_scratch(ctx->device, &base);
  if (st != HG_OK) return st;
  cudaStream_t s = ctx->stream;
  double *dmn = reinterpret_cast<double *>(base + SP_MN);
  double *dmx = reinterpret_cast<double *>(base + SP_MX);
  int2 *home = reinterpret_cast<int2 *>(base + SP_HOME);
  int32_t *bcount = reinterpret_cast<int32_t *>(base + SP_BCOUNT);
  int32_t *bstart = reinterpret_cast<int32_t *>(base + SP_BSTART);
  int32_t *bcursor = reinterpret_cast<int32_t *>(base + SP_BCURSOR);
  int32_t *items = reinterpret_cast<int32_t *>(base + SP_ITEMS);
  int32_t *cnt = reinterpret_cast<int32_t *>(base + SP_CNT);
  int32_t *off = reinterpret_cast<int32_t *>(base + SP_OFF);
  int32_t *tmp = reinterpret_cast<int32_t *>(base + SP_TMP);
  int32_t *dpairs = reinterpret_cast<int32_t *>(base + SP_PAIRS);
  uint32_t *status = reinterpret_cast<uint32_t *>(base + SP_STATUS);
  // Inputs in, counters cleared: the array keeps the previous call's contents.
  HG_CUDA_TRY(cudaMemcpyAsync(dmn, aabb_min, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s));
  HG_CUDA_TRY(cudaMemcpyAsync(dmx, aabb_max, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s));
  HG_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(uint32_t), s));
  HG_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (n + 1), s));
  const uint32_t bits = std::min<uint32_t>(table_bits(n), SP_TABLE_BITS);
  BroadArgs B;
  B.n = n;
  B.H = H;
  B.mask = (1u << bits) - 1u;
  B.mn = dmn;
  B.mx = dmx;
  if ((st = build_buckets(s, B, bcount, bstart, bcursor, items, home, tmp))) return st;
  HG_LAUNCH(kd_box_pairs<false>, blocks_for(n, 128), 128, 0, s, B, home, bstart, bcount, items,
            cnt, off, nullptr, 0, status);
  HG_CHECK_LAUNCH();
  if ((st = exclusive_scan_i32(cnt, off, n + 1, tmp, s))) return st;
  int32_t total = 0;
  uint32_t word = 0;
  HG_CUDA_TRY(cudaMemcpyAsync(&total, off + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaMemcpyAsync(&word, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  if (word & HG_STATUS_CELL_OVERFLOW)
    return fail(HG_ERR_CAPACITY, "more than 32 overlapping boxes for one box");
  if (total > SP_MAX_PAIRS)
    return fail(HG_ERR_CAPACITY, "hg_dem_candidate_pairs_static holds at most " +
                                     std::to_string(SP_MAX_PAIRS) + " pairs, found " +
                                     std::to_string(total));
  HG_LAUNCH(kd_box_pairs<true>, blocks_for(n, 128), 128, 0, s, B, home, bstart, bcount, items,
            cnt, off, dpairs, (int64_t)total, status);
  HG_CHECK_LAUNCH();
  const int64_t k = std::min<int64_t>(total, cap);
  if (k > 0)
    HG_CUDA_TRY(cudaMemcpyAsync(pairs, dpairs, sizeof(int32_t) * 2 * k, cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  *count = total;
  return HG_OK;
}
