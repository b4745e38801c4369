// Resampling of the hybrid method (ResamplingTools + CAvoidAVoid,
// hybridgrains2dnew/ResamplingTools.cpp and AvoidAvoid.cpp), host code run
// at the resampling interval on state copied from the device, after the
// zone labels (zones.cu) are updated. One call does what
// HybridGrains2DSim::updateHybridStates_poorman does between computeRZones
// and the mass-weight update (HybridGrains2DSim.cpp:327-536):
//
//   1. new grains in the reconciliation zones and new material points in the
//      reconciliation (and direct-transition) zones and in the inner
//      continuum zones, by random insertion without overlap;
//   2. their quantities: masses/volumes per hybrid cell, Gaussian-weighted
//      neighbour averages of J, be_bar, velocity and reference position
//      (or the homogenised stress and velocity), mass-weighted grid fields
//      for inner continuum points, and the mass/volume shared with their
//      neighbours;
//   3. deletion of points in discrete cells and of grains in continuum
//      cells (and of anything outside the MPM grid);
//   4. the DEM and MPM mass weights (1, 0.5 or 0 by zone) and the masses.
//
// The random stream is MT19937 in the form of hybridgrains2dnew/random.c
// (Knuth's 69069 seeding, default seed 4357, float outputs) for positions,
// and std::default_random_engine + std::normal_distribution for grain radii,
// as the reference uses them. Everything runs in the reference's order, with
// FP64 expressions in its evaluation order (this file is compiled without
// FMA contraction); results are bit-exact against the oracle.
#include "hg_internal.cuh"
#include "mpm_basis.cuh"
#include "zones_internal.cuh"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace {

// MT19937 (Matsumoto and Nishimura, 1998), with the 1998 reference code's
// seeding and single-precision output in [0, 1).
struct Mt19937 {
  static constexpr int N = 624, M = 397;
  uint32_t s[N];
  int i = N + 1; // not seeded
  void seed(uint32_t v) {
    s[0] = v;
    for (i = 1; i < N; ++i) s[i] = 69069u * s[i - 1];
  }
  uint32_t next() {
    if (i >= N) {
      if (i == N + 1) seed(4357u);
      // the twist of every word in place, in order; the index arithmetic
      // mod N split into its three ranges
      auto twist = [&](int k, int k1, int km) {
        const uint32_t y = (s[k] & 0x80000000u) | (s[k1] & 0x7fffffffu);
        s[k] = s[km] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      };
      int k = 0;
      for (; k < N - M; ++k) twist(k, k + 1, k + M);
      for (; k < N - 1; ++k) twist(k, k + 1, k + M - N);
      twist(N - 1, 0, M - 1);
      i = 0;
    }
    uint32_t y = s[i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  float uniform() { return (float)next() * 2.3283064365386963e-10f; }
  static uint32_t temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  // the state words behind the next n outputs, untempered (temper(w) of
  // each is what n calls of next() would give), a block of the state at a
  // time: the caller tempers them where it uses them
  void fill_raw(uint32_t *out, size_t n) {
    size_t k = 0;
    while (k < n) {
      if (i >= N) { // the twist of next(), undone to its raw word
        next();
        --i;
      }
      const size_t take = std::min(n - k, (size_t)(N - i));
      std::memcpy(out + k, s + i, take * sizeof(uint32_t));
      i += (int)take;
      k += take;
    }
  }
};

// uniform() of an untempered state word
inline float mt_uniform(uint32_t raw) { return (float)Mt19937::temper(raw) * 2.3283064365386963e-10f; }

inline double dist2d(double ax, double ay, double bx, double by) {
  const double dx = ax - bx, dy = ay - by;
  return std::sqrt(dx * dx + dy * dy);
}

// CUniformGridH2D (uniformgrid.cpp) with points registered by the cell that
// holds them: per-cell id lists in CSR form, each in increasing id order (the
// order in which the reference appends them).
struct CellLists {
  double mn[2] = {0, 0}, cw = 1.0;
  unsigned res[2] = {1, 1};
  std::vector<int> start, ids;
  struct Span {
    const int *b, *e;
    const int *begin() const { return b; }
    const int *end() const { return e; }
    size_t size() const { return (size_t)(e - b); }
  };
  void reset(double x0, double y0, unsigned rx, unsigned ry, double w) {
    mn[0] = x0;
    mn[1] = y0;
    res[0] = std::max(rx, 1u);
    res[1] = std::max(ry, 1u);
    cw = w;
    start.assign((size_t)res[0] * res[1] + 1, 0);
    ids.clear();
  }
  void cell(double x, double y, unsigned &i, unsigned &j) const {
    const double u = (x - mn[0]) / cw, v = (y - mn[1]) / cw;
    i = (unsigned)std::max<int>(0, std::min<int>((int)res[0] - 1, (int)std::floor(u)));
    j = (unsigned)std::max<int>(0, std::min<int>((int)res[1] - 1, (int)std::floor(v)));
  }
  // n points at xy[stride k], xy[stride k + 1] with ids 0 .. n-1 (a counting
  // sort by cell, stable in id order)
  void add_points(const double *xy, int stride, size_t n) {
    std::vector<int> c(n);
    for (size_t k = 0; k < n; ++k) {
      unsigned i, j;
      cell(xy[stride * k], xy[stride * k + 1], i, j);
      c[k] = (int)((size_t)j * res[0] + i);
      start[c[k] + 1]++;
    }
    for (size_t q = 0; q + 1 < start.size(); ++q) start[q + 1] += start[q];
    ids.assign(n, 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (size_t k = 0; k < n; ++k) ids[fill[c[k]]++] = (int)k;
  }
  Span at(unsigned i, unsigned j) const {
    if (i >= res[0] || j >= res[1]) return Span{nullptr, nullptr};
    const size_t c = (size_t)j * res[0] + i;
    return Span{ids.data() + start[c], ids.data() + start[c + 1]};
  }
};

} // namespace

struct hg_resampler {
  hg_resampler_desc d{};
  double grid_h = 0.0; // cell width of the interpolation grids, (max - min) / n
  Mt19937 mt;
  std::default_random_engine gen;
  std::normal_distribution<double> radius_dist;
  int test_id = 100;
  // MPM points (MaterialPoints)
  std::vector<double> q0, q, v, m, vol, m0, vol0, w, hl, be, J;
  std::vector<int32_t> jh;
  std::vector<uint8_t> kin;
  // DEM bodies (RigidBody2DState)
  std::vector<double> dq0, dq, dv, dr, M0, dw;
  std::vector<uint8_t> fixed;
  std::vector<int32_t> dem_map; // old (after insertion) -> new index, -1 deleted
  // homogenised fields per node: stress 4 (column-major), velocity 2
  std::vector<double> hs, hv;
  hg_resampler_stats stats{};
};

namespace {

using Box = hg_zones::Box;

size_t npoints(const hg_resampler &r) { return r.m.size(); }
size_t nbodies(const hg_resampler &r) { return r.dr.size(); }

// Candidate search of fill_regions. A sample conflicts with a body when
// their centres are closer than 0.97 (r_body + r_sample); whether one does
// is all the reference's search (AvoidAvoid.cpp:133-165, bodies registered in
// every cell their boxes cover, each tested once per sample) decides, so any
// search that reaches every body within that distance decides the same.
// Bodies of radius at most cw / 2 are kept by the cell of their centre: the
// ones present at the start contiguously per cell (centre and radius
// inline), the samples accepted since in per-cell lists. A body within
// conflict distance of a sample of radius r lies within 0.97 (cw / 2 + r) of
// it, so the cells within ceil((cw / 2 + r) / cw) of the sample's hold it
// (the 3 x 3 around it when r <= cw / 2). Wider bodies are tested by every
// sample. Squared distances decide outside a 1e-12 relative band around the
// limit; inside it the reference's expression sqrt(dx^2 + dy^2) < 0.97
// (r_body + r) does, on the same dx and dy.
inline bool conflicts(double bx, double by, double br, double x, double y, double r) {
  const double dx = bx - x, dy = by - y;
  const double d2 = dx * dx + dy * dy, lim = (br + r) * 0.97, l2 = lim * lim;
  if (d2 > l2 * (1.0 + 1.0e-12)) return false;
  if (d2 < l2 * (1.0 - 1.0e-12)) return true;
  return dist2d(bx, by, x, y) < lim;
}

struct FillGrid {
  double x0 = 0, y0 = 0, cw = 1;
  int nx = 1, ny = 1;
  std::vector<int> start;              // per cell, into the initial bodies
  std::vector<double> bx, by, br;      // initial bodies in cell order
  std::vector<double> ix, iy, ir;      // initial bodies wider than cw / 2
  std::vector<int> head, next;         // samples accepted since: per-cell lists
  std::vector<double> sx, sy, sr;
  std::vector<double> wx, wy, wr;      // accepted samples wider than cw / 2
  int cx(double x) const { return std::max(0, std::min(nx - 1, (int)std::floor((x - x0) / cw))); }
  int cy(double y) const { return std::max(0, std::min(ny - 1, (int)std::floor((y - y0) / cw))); }
  void add_sample(double x, double y, double r) {
    if (r > 0.5 * cw) {
      wx.push_back(x);
      wy.push_back(y);
      wr.push_back(r);
      return;
    }
    const int c = cy(y) * nx + cx(x);
    next.push_back(head[c]);
    head[c] = (int)sx.size();
    sx.push_back(x);
    sy.push_back(y);
    sr.push_back(r);
  }
  // the cells a body within conflict distance of (x, y, r) can be in
  template <typename F>
  bool any_cell(double x, double y, double r, F f) const {
    const int reach = (int)std::ceil((0.5 * cw + r) / cw);
    const int i = cx(x), j = cy(y);
    // the sample's own cell first: most conflicts are found there
    if (f(j * nx + i)) return true;
    const int i0 = std::max(0, i - reach), i1 = std::min(nx - 1, i + reach);
    const int j0 = std::max(0, j - reach), j1 = std::min(ny - 1, j + reach);
    for (int jj = j0; jj <= j1; ++jj)
      for (int ii = i0; ii <= i1; ++ii)
        if ((ii != i || jj != j) && f(jj * nx + ii)) return true;
    return false;
  }
  bool conflict_initial(double x, double y, double r) const {
    for (size_t k = 0; k < ix.size(); ++k)
      if (conflicts(ix[k], iy[k], ir[k], x, y, r)) return true;
    return any_cell(x, y, r, [&](int c) {
      for (int k = start[c]; k < start[c + 1]; ++k)
        if (conflicts(bx[k], by[k], br[k], x, y, r)) return true;
      return false;
    });
  }
  bool conflict_accepted(double x, double y, double r) const {
    for (size_t k = 0; k < wx.size(); ++k)
      if (conflicts(wx[k], wy[k], wr[k], x, y, r)) return true;
    return any_cell(x, y, r, [&](int c) {
      for (int k = head[c]; k >= 0; k = next[k])
        if (conflicts(sx[k], sy[k], sr[k], x, y, r)) return true;
      return false;
    });
  }
};

// t advanced k times by "if (++t == 0) t = 1": the stamps run through
// 1 .. 2^32 - 1 in a cycle, and 0 (not yet stamped) comes before 1.
inline void advance_test_id(int &t, uint64_t k) {
  if (k == 0) return;
  const uint64_t cycle = 0xFFFFFFFFull; // stamps 1 .. 2^32 - 1
  const uint64_t u = (uint32_t)t;
  // index in the cycle: stamp 1 is 0, stamp 0 (the start) is -1
  const uint64_t idx = u == 0 ? (k - 1) % cycle : (u - 1 + k % cycle) % cycle;
  t = (int)(uint32_t)(idx + 1);
}

// The search grid of fill_trials over the bodies (px, py, rad), for samples
// in [g0x, g1x] x [g0y, g1y], with cells 2 rc wide.
void build_fill_grid(FillGrid &grid, double g0x, double g0y, double g1x, double g1y, double rc,
                     const std::vector<double> &px, const std::vector<double> &py,
                     const std::vector<double> &rad) {
  // scratch kept between calls (the interval repeats with similar sizes, and
  // fresh pages would be faulted in on every call)
  static thread_local std::vector<int> tl_cell_of;
  std::vector<int> &cell_of = tl_cell_of;
  grid.bx.clear();
  grid.by.clear();
  grid.br.clear();
  grid.ix.clear();
  grid.iy.clear();
  grid.ir.clear();
  grid.next.clear();
  grid.sx.clear();
  grid.sy.clear();
  grid.sr.clear();
  grid.wx.clear();
  grid.wy.clear();
  grid.wr.clear();
  grid.x0 = g0x;
  grid.y0 = g0y;
  grid.cw = 2.0 * rc;
  grid.nx = std::max(1, (int)std::ceil((g1x - g0x) / grid.cw));
  grid.ny = std::max(1, (int)std::ceil((g1y - g0y) / grid.cw));
  const size_t ncell = (size_t)grid.nx * grid.ny;
  // counting sort of the initial bodies by the cell of their centre. A body
  // wholly outside the grid's extent cannot conflict with a sample (samples
  // lie in the regions, six mean radii inside that extent); the reference's
  // grid leaves it out too.
  // cell of each body's centre (-1: outside the extent, -2: wider than
  // cw / 2), over host threads; then a counting sort
  cell_of.assign(px.size(), -1);
  hg::host_parallel(px.size(), 16384, [&](size_t b0, size_t b1) {
    for (size_t b = b0; b < b1; ++b) {
      if (px[b] + rad[b] < g0x || px[b] - rad[b] > g1x || py[b] + rad[b] < g0y ||
          py[b] - rad[b] > g1y)
        continue;
      cell_of[b] = rad[b] > 0.5 * grid.cw ? -2 : grid.cy(py[b]) * grid.nx + grid.cx(px[b]);
    }
  });
  grid.start.assign(ncell + 1, 0);
  for (size_t b = 0; b < px.size(); ++b) {
    if (cell_of[b] == -2) {
      grid.ix.push_back(px[b]);
      grid.iy.push_back(py[b]);
      grid.ir.push_back(rad[b]);
    } else if (cell_of[b] >= 0) {
      grid.start[cell_of[b] + 1]++;
    }
  }
  for (size_t c = 0; c < ncell; ++c) grid.start[c + 1] += grid.start[c];
  const int nb = grid.start[ncell];
  grid.bx.resize(nb);
  grid.by.resize(nb);
  grid.br.resize(nb);
  {
    std::vector<int> fill(grid.start.begin(), grid.start.end() - 1);
    for (size_t b = 0; b < px.size(); ++b) {
      if (cell_of[b] < 0) continue;
      const int k = fill[cell_of[b]]++;
      grid.bx[k] = px[b];
      grid.by[k] = py[b];
      grid.br[k] = rad[b];
    }
  }
  grid.head.assign(ncell, -1);
}

// The trials of CAvoidAVoid::avoidAVoid with randomFillRegion
// (AvoidAvoid.cpp:103-183) over the regions, against the bodies of the grid
// (built over the bodies present, plus the samples accepted since): accepted
// samples are appended to (px, py, rad) and added to the grid.
// (fixed_r > 0: every sample has that radius and the sampler is not called;
// words: the trials' 2 x 16 x regions position words drawn already, in
// their order in R.mt's stream, the test id then advanced by the caller)
template <typename Sampler>
hg_status fill_trials(hg_resampler &R, FillGrid &grid, const std::vector<Box> &regions,
                      std::vector<double> &px, std::vector<double> &py,
                      std::vector<double> &rad, Sampler sampler, double fixed_r = -1.0,
                      const uint32_t *words = nullptr) {
  if (regions.empty()) return HG_OK;
  static thread_local std::vector<double> tl_tx, tl_ty, tl_tr;
  static thread_local std::vector<uint8_t> tl_hit;
  static thread_local std::vector<uint32_t> tl_raw;
  std::vector<double> &tx = tl_tx, &ty = tl_ty, &tr = tl_tr;
  std::vector<uint8_t> &hit = tl_hit;
  std::vector<uint32_t> &raw = tl_raw;
  // 16 trials per region in the reference's order. Neither the positions
  // (R.mt) nor the radii (the sampler's own engine) depend on which trials
  // are accepted, so all are drawn first: the position words in one run of
  // the generator, converted over host threads, the radii in trial order. A
  // trial is accepted when it conflicts neither with the bodies present at
  // the start (tested for all trials at once, over host threads) nor with
  // the trials accepted before it (tested in trial order).
  const size_t T = 16 * regions.size();
  tx.resize(T);
  ty.resize(T);
  tr.resize(T);
  const uint32_t *rw = words;
  if (!rw) {
    raw.resize(2 * T);
    R.mt.fill_raw(raw.data(), 2 * T);
    rw = raw.data();
  }
  if (fixed_r > 0.0) {
    std::fill(tr.begin(), tr.begin() + T, fixed_r);
  } else {
    for (size_t t = 0; t < T; ++t) {
      const hg_status st = sampler(tr[t]);
      if (st != HG_OK) return st;
    }
  }
  hit.resize(T);
  hg::host_parallel(T, 4096, [&](size_t b, size_t e) {
    for (size_t k = b; k < e; ++k) {
      const Box &reg = regions[k / 16];
      const double dx = reg.b[2] - reg.b[0], dy = reg.b[3] - reg.b[1];
      tx[k] = (double)mt_uniform(rw[2 * k]) * dx + reg.b[0];
      ty[k] = (double)mt_uniform(rw[2 * k + 1]) * dy + reg.b[1];
      hit[k] = grid.conflict_initial(tx[k], ty[k], tr[k]) ? 1 : 0;
    }
  });
  for (size_t k = 0; k < T; ++k) {
    if (hit[k] || grid.conflict_accepted(tx[k], ty[k], tr[k])) continue;
    px.push_back(tx[k]);
    py.push_back(ty[k]);
    rad.push_back(tr[k]);
    grid.add_sample(tx[k], ty[k], tr[k]);
  }
  // the reference's mailbox stamp advances once per test, through 1 .. 2^32 - 1
  // (0 is skipped on the wrap)
  if (!words) advance_test_id(R.test_id, T);
  return HG_OK;
}

// The bounding box of the regions, widened by six mean radii.
void regions_extent(const std::vector<Box> &regions, double mean_r, double e[4]) {
  double lo[2] = {regions[0].b[0], regions[0].b[1]}, up[2] = {regions[0].b[2], regions[0].b[3]};
  for (size_t k = 1; k < regions.size(); ++k) {
    lo[0] = std::min(lo[0], regions[k].b[0]);
    lo[1] = std::min(lo[1], regions[k].b[1]);
    up[0] = std::max(up[0], regions[k].b[2]);
    up[1] = std::max(up[1], regions[k].b[3]);
  }
  e[0] = lo[0] - 6.0 * mean_r;
  e[1] = lo[1] - 6.0 * mean_r;
  e[2] = up[0] + 6.0 * mean_r;
  e[3] = up[1] + 6.0 * mean_r;
}

// CAvoidAVoid::avoidAVoid with randomFillRegion (AvoidAvoid.cpp:103-183):
// bodies (px, py, rad) grow by the accepted samples, whose radii are at most
// r_max.
template <typename Sampler>
hg_status fill_regions(hg_resampler &R, const std::vector<Box> &regions, double mean_r,
                       double r_max, std::vector<double> &px, std::vector<double> &py,
                       std::vector<double> &rad, Sampler sampler,
                       const uint32_t *words = nullptr) {
  if (regions.empty()) return HG_OK;
  double e[4];
  regions_extent(regions, mean_r, e);
  // cells twice the largest radius of the samples and of the bodies up to
  // four mean radii (wider ones go to the list every sample scans)
  double rc = r_max;
  for (size_t b = 0; b < px.size(); ++b)
    if (rad[b] > rc && rad[b] <= 4.0 * mean_r) rc = rad[b];
  static thread_local FillGrid tl_grid;
  build_fill_grid(tl_grid, e[0], e[1], e[2], e[3], rc, px, py, rad);
  return fill_trials(R, tl_grid, regions, px, py, rad, sampler, -1.0, words);
}

// avoidAVoidMPMparticlesInsideZonesWithTentativeQuantities
// (ResamplingTools.cpp:58-104): returns the count before insertion. grid:
// the search grid over the points, shared by the interval's point
// insertions (a sample of one insertion is a body of the next: it is one of
// the grid's accepted samples, which every later trial tests).
hg_status insert_points(hg_resampler &R, const std::vector<Box> &zones, int64_t &before,
                        FillGrid &grid, const uint32_t *words) {
  const double rp = 0.5 * R.d.initial_particle_size;
  const size_t n = npoints(R);
  before = (int64_t)n;
  std::vector<double> px, py, rad;
  const hg_status st = fill_trials(R, grid, zones, px, py, rad, [&](double &r) -> hg_status {
    r = rp;
    return HG_OK;
  }, rp, words);
  if (st != HG_OK) return st;
  const double hl0 = R.d.initial_particle_size * 0.5;
  for (size_t p = 0; p < px.size(); ++p) { // addMaterialPoint, MaterialPoints.cpp:439-467
    R.q0.push_back(px[p]);
    R.q0.push_back(py[p]);
    R.q.push_back(px[p]);
    R.q.push_back(py[p]);
    R.v.push_back(0.0);
    R.v.push_back(0.0);
    R.m.push_back(0.0);
    R.vol.push_back(0.0);
    R.m0.push_back(0.0);
    R.vol0.push_back(0.0);
    R.w.push_back(1.0);
    R.hl.push_back(hl0);
    const double I4[4] = {1.0, 0.0, 0.0, 1.0};
    R.be.insert(R.be.end(), I4, I4 + 4);
    R.J.push_back(1.0);
    R.jh.push_back(0);
    R.kin.push_back(0);
  }
  R.stats.points_inserted += (int64_t)px.size();
  return HG_OK;
}

// avoidAVoidDEMparticlesInsideZonesWithTentativeQuantities
// (ResamplingTools.cpp:106-196) with randomRadiusSampler (:19-26).
hg_status insert_grains(hg_resampler &R, const std::vector<Box> &zones, int64_t &before,
                        const uint32_t *words) {
  const size_t n = nbodies(R);
  before = (int64_t)n;
  std::vector<double> px(n), py(n), rad(R.dr);
  for (size_t b = 0; b < n; ++b) {
    px[b] = R.dq[3 * b];
    py[b] = R.dq[3 * b + 1];
  }
  double r_mean = R.d.dem_r_mean;
  const double lo = R.d.dem_r_mean - 2.0 * R.d.dem_r_std, hi = R.d.dem_r_mean + 2.0 * R.d.dem_r_std;
  bool unset = false;
  if (R.d.dem_r_mean < 0.0) { // the first radius, without spread
    if (n == 0) return hg::fail(HG_ERR_INVALID_ARGUMENT, "no grain radius to sample from");
    r_mean = rad[0];
    R.radius_dist = std::normal_distribution<double>(rad[0], 0.0);
    unset = true;
  }
  const double r_max = unset ? rad[0] : hi;
  const hg_status st = fill_regions(R, zones, r_mean, r_max, px, py, rad,
                                   [&](double &r) -> hg_status {
    if (unset) {
      // the reference's rejection bounds stay at the unset mean and would
      // never accept: take the sampled radius as is
      r = R.radius_dist(R.gen);
      return HG_OK;
    }
    r = -1.0e33;
    for (int k = 0; r < lo || r > hi; ++k) {
      if (k == 1000000) return hg::fail(HG_ERR_INVALID_ARGUMENT, "grain radius sampler does not accept");
      r = R.radius_dist(R.gen);
    }
    return HG_OK;
  }, words);
  if (st != HG_OK) return st;
  const double pi = 3.14159265358979323846;
  for (size_t b = n; b < px.size(); ++b) { // RigidBody2DState::addBodies
    const double r = rad[b];
    const double m = R.d.rho_dem * pi * r * r; // CircleGeometry::massAndInertia
    const double I = 0.5 * m * r * r;
    const double q3[3] = {px[b], py[b], 0.0}, z3[3] = {0.0, 0.0, 0.0}, m3[3] = {m, m, I};
    R.dq.insert(R.dq.end(), q3, q3 + 3);
    R.dq0.insert(R.dq0.end(), q3, q3 + 3);
    R.dv.insert(R.dv.end(), z3, z3 + 3);
    R.dr.push_back(r);
    R.M0.insert(R.M0.end(), m3, m3 + 3);
    R.dw.push_back(1.0);
    R.fixed.push_back(0);
  }
  R.stats.grains_inserted += (int64_t)(px.size() - n);
  return HG_OK;
}

// Uniform grids over the MPM cells with points and grains as points
// (ZoneTools::setupUniformGridElementsAsPoints, ZoneTools.cpp:800-827).
void point_grids(const hg_resampler &R, CellLists &cont, CellLists &disc) {
  const hg_zones_desc &zd = R.d.zones;
  cont.reset(zd.mpm_grid_min[0], zd.mpm_grid_min[1], zd.mpm_cells[0], zd.mpm_cells[1],
             zd.mpm_cell_width);
  disc.reset(zd.mpm_grid_min[0], zd.mpm_grid_min[1], zd.mpm_cells[0], zd.mpm_cells[1],
             zd.mpm_cell_width);
  cont.add_points(R.q.data(), 2, npoints(R));
  disc.add_points(R.dq.data(), 3, nbodies(R));
}

template <typename F>
void for_range(const CellLists &g, double x0, double y0, double x1, double y1, F f) {
  unsigned i0, j0, i1, j1;
  g.cell(x0, y0, i0, j0);
  g.cell(x1, y1, i1, j1);
  for (unsigned j = j0; j <= j1; ++j)
    for (unsigned i = i0; i <= i1; ++i)
      for (int id : g.at(i, j)) f(id);
}

// Node range of a stencil as the reference iterates it: its bounds are cast
// to unsigned, so a stencil starting left of or below the grid (x - hl <
// grid min for uGIMP) runs no iteration at all; nodes past the last one are
// skipped (the reference would read past its arrays there).
inline bool stencil_range(int a0, int a1, int last, int &b0, int &b1) {
  if (a0 < 0) return false;
  b0 = a0;
  b1 = std::min(a1, last);
  return b0 <= b1;
}

// Interpolation of a node field with the MPM basis at half width hl
// (computeStencil / weight over the physics grid).
void interp_nodes(const hg_resampler &R, double x, double y, double hl, double gmin_x,
                  double gmin_y, double h, int nx, const std::vector<double> &field, int len,
                  double *out) {
  for (int c = 0; c < len; ++c) out[c] = 0.0;
  const int ny = R.d.zones.mpm_cells[1];
  int x0, y0, x1, y1, i0, i1, j0, j1;
  hg::stencil64(R.d.basis, x, y, hl, gmin_x, gmin_y, h, x0, y0, x1, y1);
  if (!stencil_range(y0, y1, ny, j0, j1) || !stencil_range(x0, x1, nx, i0, i1)) return;
  for (int iy = j0; iy <= j1; ++iy)
    for (int ix = i0; ix <= i1; ++ix) {
      const double wgt = hg::weight64(R.d.basis, x, y, hl, ix, iy, gmin_x, gmin_y, h);
      const size_t node = (size_t)iy * (nx + 1) + ix;
      for (int c = 0; c < len; ++c) out[c] += wgt * field[node * len + c];
    }
}

// 2x2 determinant in column-major storage (a00, a10, a01, a11)
inline double det2(const double *a) { return a[0] * a[3] - a[1] * a[2]; }

// ConstitutiveModel::computeStrainFromCauchyStress (ConstitutiveModel.cpp:99-117)
void strain_from_stress(const double *s, double kappa, double mu, double &J, double *be) {
  const double T = s[0] + s[3];
  J = 0.5 * (T / kappa + std::sqrt((T * T) / (kappa * kappa) + 4.0));
  double dev[4] = {s[0] - T * 1.0 / 2.0, s[1] - T * 0.0 / 2.0, s[2] - T * 0.0 / 2.0,
                   s[3] - T * 1.0 / 2.0};
  for (int c = 0; c < 4; ++c) dev[c] = J * dev[c] / mu;
  const double t = std::sqrt(1.0 - det2(dev));
  be[0] = dev[0] + t * 1.0;
  be[1] = dev[1] + t * 0.0;
  be[2] = dev[2] + t * 0.0;
  be[3] = dev[3] + t * 1.0;
}

// determineMPMQuantitiesForHybridZones (ResamplingTools.cpp:616-639) with
// reassignMassAndVolumesForHybridAndNewlyGeneratedContinuumZone (:379-400)
// and reassignJVelAndBebarForHybridMaterialPoint (:402-612).
void hybrid_point_quantities(hg_resampler &R, const std::vector<Box> &zones, int64_t before,
                             int64_t after, int64_t grains_before, const CellLists &cont,
                             const CellLists &disc) {
  const hg_zones_desc &zd = R.d.zones;
  const double cell_volume = zd.mpm_cell_width * zd.mpm_cell_width;
  const double mass_per_cell = R.d.material_density * cell_volume;
  for (const Box &z : zones) {
    const CellLists::Span ids = cont.at((unsigned)z.c[0], (unsigned)z.c[1]);
    const int n = (int)ids.size();
    for (int id : ids) {
      R.m0[id] = mass_per_cell / n;
      R.vol0[id] = cell_volume / n;
    }
  }
  const double size = R.d.initial_particle_size;
  const double sigma = 0.5 * size, max_dist = 3.0 * size;
  const double hh = zd.mpm_cell_width * 0.25;
  // each inserted point reads only the points and grains that were there
  // before the insertion and writes only its own entries: over host threads
  hg::host_parallel((size_t)(after - before), 256, [&](size_t pb, size_t pe) {
  for (int64_t p = before + (int64_t)pb; p < before + (int64_t)pe; ++p) {
    const double x = R.q[2 * p], y = R.q[2 * p + 1];
    double vs[2] = {0, 0}, q0s[2] = {0, 0}, Js = 0.0, bes[4] = {0, 0, 0, 0}, ws = 0.0;
    int nn = 0;
    for_range(cont, x - max_dist, y - max_dist, x + max_dist, y + max_dist, [&](int id) {
      if (id >= before) return;
      const double d = dist2d(R.q[2 * id], R.q[2 * id + 1], x, y);
      if (d <= max_dist) {
        const double wgt = std::exp(-(d * d) / (2.0 * sigma * sigma));
        vs[0] += R.v[2 * id] * wgt;
        vs[1] += R.v[2 * id + 1] * wgt;
        q0s[0] += R.q0[2 * id] * wgt;
        q0s[1] += R.q0[2 * id + 1] * wgt;
        Js += R.J[id] * wgt;
        for (int c = 0; c < 4; ++c) bes[c] += R.be[4 * id + c] * wgt;
        ws += wgt;
        ++nn;
      }
    });
    double stress[4] = {0, 0, 0, 0}, hvel[2] = {0, 0};
    if (R.d.homogenize_stress)
      interp_nodes(R, x, y, hh, zd.mpm_grid_min[0], zd.mpm_grid_min[1], zd.mpm_cell_width,
                   zd.mpm_cells[0], R.hs, 4, stress);
    if (R.d.homogenize_velocity)
      interp_nodes(R, x, y, hh, zd.mpm_grid_min[0], zd.mpm_grid_min[1], zd.mpm_cell_width,
                   zd.mpm_cells[0], R.hv, 2, hvel);
    double Jn, ben[4];
    if (nn == 0) {
      Jn = 1.0;
      ben[0] = 1.0, ben[1] = 0.0, ben[2] = 0.0, ben[3] = 1.0;
    } else {
      Jn = Js / ws;
      for (int c = 0; c < 4; ++c) ben[c] = bes[c] / ws;
      const double sd = std::sqrt(det2(ben));
      for (int c = 0; c < 4; ++c) ben[c] = ben[c] / sd;
    }
    for_range(disc, x - max_dist, y - max_dist, x + max_dist, y + max_dist, [&](int id) {
      if (id >= grains_before) return;
      const double d = dist2d(R.dq[3 * id], R.dq[3 * id + 1], x, y);
      if (d <= max_dist) {
        const double wgt = std::exp(-(d * d) / (2.0 * sigma * sigma));
        vs[0] += R.dv[3 * id] * wgt;
        vs[1] += R.dv[3 * id + 1] * wgt;
        q0s[0] += R.dq0[3 * id] * wgt;
        q0s[1] += R.dq0[3 * id + 1] * wgt;
        ws += wgt;
      }
    });
    double vn[2], q0n[2];
    if (ws == 0.0) {
      vn[0] = vn[1] = 0.0;
      q0n[0] = x;
      q0n[1] = y;
    } else {
      vn[0] = vs[0] / ws;
      vn[1] = vs[1] / ws;
      q0n[0] = q0s[0] / ws;
      q0n[1] = q0s[1] / ws;
    }
    R.q0[2 * p] = q0n[0];
    R.q0[2 * p + 1] = q0n[1];
    R.v[2 * p] = R.d.homogenize_velocity ? hvel[0] : vn[0];
    R.v[2 * p + 1] = R.d.homogenize_velocity ? hvel[1] : vn[1];
    if (R.d.homogenize_stress) {
      strain_from_stress(stress, R.d.kappa, R.d.mu, Jn, ben);
      R.J[p] = Jn;
    } else {
      R.J[p] = R.d.newly_inserted_continuum_stress_free ? 1.0 : Jn;
    }
    for (int c = 0; c < 4; ++c) R.be[4 * p + c] = ben[c];
  }
  });
}

// determineDEMQuantitiesForHybridZones (ResamplingTools.cpp:646-725)
void grain_quantities(hg_resampler &R, int64_t before, int64_t after, int64_t points_before,
                      const CellLists &cont, const CellLists &disc) {
  const double sigma = R.d.dem_r_mean, max_dist = 6.0 * R.d.dem_r_mean;
  // each inserted grain reads only the bodies and points there before the
  // insertion: over host threads
  hg::host_parallel((size_t)(after - before), 256, [&](size_t gb, size_t ge) {
  for (int64_t b = before + (int64_t)gb; b < before + (int64_t)ge; ++b) {
    const double x = R.dq[3 * b], y = R.dq[3 * b + 1];
    double vs[3] = {0, 0, 0}, q0s[3] = {0, 0, 0}, ws = 0.0;
    for_range(disc, x - max_dist, y - max_dist, x + max_dist, y + max_dist, [&](int id) {
      if (id >= before) return;
      const double d = dist2d(R.dq[3 * id], R.dq[3 * id + 1], x, y);
      if (d <= max_dist) {
        const double wgt = std::exp(-(d * d) / (2.0 * sigma * sigma));
        for (int c = 0; c < 3; ++c) {
          vs[c] += R.dv[3 * id + c] * wgt;
          q0s[c] += R.dq0[3 * id + c] * wgt;
        }
        ws += wgt;
      }
    });
    for_range(cont, x - max_dist, y - max_dist, x + max_dist, y + max_dist, [&](int id) {
      if (id >= points_before) return;
      const double d = dist2d(R.q[2 * id], R.q[2 * id + 1], x, y);
      if (d <= max_dist) {
        const double wgt = std::exp(-(d * d) / (2.0 * sigma * sigma));
        vs[0] += R.v[2 * id] * wgt;
        vs[1] += R.v[2 * id + 1] * wgt;
        vs[2] += 0.0 * wgt;
        q0s[0] += R.q0[2 * id] * wgt;
        q0s[1] += R.q0[2 * id + 1] * wgt;
        q0s[2] += 0.0 * wgt;
        ws += wgt;
      }
    });
    if (ws == 0.0) {
      for (int c = 0; c < 3; ++c) R.dv[3 * b + c] = 0.0;
      R.dq0[3 * b] = x;
      R.dq0[3 * b + 1] = y;
      R.dq0[3 * b + 2] = 0.0;
    } else {
      for (int c = 0; c < 3; ++c) {
        R.dv[3 * b + c] = vs[c] / ws;
        R.dq0[3 * b + c] = q0s[c] / ws;
      }
    }
  }
  });
}

// Mass-weighted node fields of the first n points (Grid::rasterizeMass +
// rasterizeMassWeightedValues* + normalizationByMass, Grid.cpp:148-348) for
// J, velocity and be_bar together: the reference builds each field in a pass
// of its own with the same stencils, weights and node mass; one pass over
// the points accumulates every field in the same per-node order, so each
// sum is bit for bit the separate pass's.
struct NodeField {
  int len;
  const std::vector<double> *vals;
  const double *dflt;
  std::vector<double> *out;
};

void mass_weighted_fields(const hg_resampler &R, int64_t n, NodeField *f, int nf) {
  const hg_zones_desc &zd = R.d.zones;
  const int nx = zd.mpm_cells[0], ny = zd.mpm_cells[1];
  const size_t nn = (size_t)(nx + 1) * (ny + 1);
  // (scratch kept between calls)
  static thread_local std::vector<double> tl_mass;
  std::vector<double> &mass = tl_mass;
  mass.assign(nn, 0.0);
  for (int k = 0; k < nf; ++k) f[k].out->assign(nn * f[k].len, 0.0);
  const double h1 = R.hl.empty() ? 0.0 : R.hl[0];
  // the node range of every point's stencil (empty: j0 > j1)
  static thread_local std::vector<std::array<int, 4>> tl_range;
  std::vector<std::array<int, 4>> &range = tl_range;
  range.resize((size_t)n);
  hg::host_parallel((size_t)n, 4096, [&](size_t b, size_t e) {
    for (size_t p = b; p < e; ++p) {
      int x0, y0, x1, y1, i0, i1, j0, j1;
      hg::stencil64(R.d.basis, R.q[2 * p], R.q[2 * p + 1], h1, zd.mpm_grid_min[0],
                    zd.mpm_grid_min[1], R.grid_h, x0, y0, x1, y1);
      if (!stencil_range(y0, y1, ny, j0, j1) || !stencil_range(x0, x1, nx, i0, i1))
        range[p] = {0, -1, 0, -1};
      else
        range[p] = {i0, i1, j0, j1};
    }
  });
  // node rows split over host threads in bands of about equal work (the
  // stencil rows the points put on them: the points fill part of the grid);
  // each thread walks the points in order, so every node sums its points in
  // the reference's order
  const size_t workers = std::max<size_t>(1, std::min(hg::host_workers(), (size_t)ny + 1));
  // (rows j0 .. j1 <= ny: +w at j0 + 1, -w at j1 + 2 <= ny + 2)
  std::vector<int64_t> work((size_t)ny + 3, 0);
  for (int64_t p = 0; p < n; ++p)
    if (range[p][2] <= range[p][3]) {
      const int64_t w = range[p][1] - range[p][0] + 1;
      work[range[p][2] + 1] += w;
      work[range[p][3] + 2] -= w;
    }
  // work per row, then its running sum
  for (size_t j = 1; j < work.size(); ++j) work[j] += work[j - 1];
  for (size_t j = 1; j < work.size(); ++j) work[j] += work[j - 1];
  std::vector<size_t> band(workers + 1, (size_t)ny + 1);
  band[0] = 0;
  for (size_t t = 1, j = 0; t < workers; ++t) {
    const int64_t goal = (int64_t)((double)work[ny + 1] * (double)t / (double)workers);
    while (j < (size_t)ny + 1 && work[j] < goal) ++j;
    band[t] = std::max(j, band[t - 1]);
  }
  hg::host_pool_run(workers, [&](size_t t) {
    const size_t rb = band[t], re = band[t + 1];
    if (rb >= re) return;
    for (int64_t p = 0; p < n; ++p) {
      const std::array<int, 4> &r = range[p];
      const int j0 = std::max(r[2], (int)rb), j1 = std::min(r[3], (int)re - 1);
      if (j0 > j1) continue;
      const double x = R.q[2 * p], y = R.q[2 * p + 1];
      for (int iy = j0; iy <= j1; ++iy)
        for (int ix = r[0]; ix <= r[1]; ++ix) {
          const double wgt = hg::weight64(R.d.basis, x, y, h1, ix, iy, zd.mpm_grid_min[0],
                                          zd.mpm_grid_min[1], R.grid_h);
          const size_t node = (size_t)iy * (nx + 1) + ix;
          mass[node] += wgt * R.m[p];
          for (int k = 0; k < nf; ++k) {
            const int len = f[k].len;
            const double *v = f[k].vals->data() + (size_t)p * len;
            double *o = f[k].out->data() + node * len;
            for (int c = 0; c < len; ++c) o[c] += wgt * R.m[p] * v[c];
          }
        }
    }
  });
  hg::host_parallel(nn, 4096, [&](size_t b, size_t e) {
    for (int k = 0; k < nf; ++k) {
      const int len = f[k].len;
      double *o = f[k].out->data();
      for (size_t node = b; node < e; ++node) {
        if (mass[node] > 0.0) {
          for (int c = 0; c < len; ++c) o[node * len + c] /= mass[node];
        } else {
          for (int c = 0; c < len; ++c) o[node * len + c] = f[k].dflt[c];
        }
      }
    }
  });
}

// determineMPMQuantitiesForInnerContinuumZones (ResamplingTools.cpp:353-377)
// with computeFieldsForInterpolation (:276-333), gatherMassAndVolume
// (:198-274) and reassignJVelAndBebarForInternalMaterialPoint (:335-366).
void inner_point_quantities(hg_resampler &R, int64_t before, int64_t after, const CellLists &cont) {
  const hg_zones_desc &zd = R.d.zones;
  if (after <= before) return; // no inner point inserted: nothing to assign
  // node fields kept between calls (fresh pages would be faulted in on
  // every call)
  static thread_local std::vector<double> tl_fJ, tl_fv, tl_fb;
  std::vector<double> &fJ = tl_fJ, &fv = tl_fv, &fb = tl_fb;
  const double dJ[1] = {1.0}, dv[2] = {0.0, 0.0}, db[4] = {1.0, 0.0, 0.0, 1.0};
  NodeField fields[3] = {{1, &R.J, dJ, &fJ}, {2, &R.v, dv, &fv}, {4, &R.be, db, &fb}};
  mass_weighted_fields(R, before, fields, 3);
  const double size = R.d.initial_particle_size;
  const double sigma = 0.5 * size, rr = 2.0 * size;
  for (int64_t i = before; i < after; ++i) { // gatherMassAndVolume
    const double x = R.q[2 * i], y = R.q[2 * i + 1];
    double tm = 0.0, tv = 0.0, ws = 0.0, q0s[2] = {0, 0};
    std::vector<int> nb;
    for_range(cont, x - rr, y - rr, x + rr, y + rr, [&](int id) {
      if (id >= i) return;
      const double ex = x - R.q[2 * id], ey = y - R.q[2 * id + 1];
      const double d2 = ex * ex + ey * ey;
      if (d2 < rr * rr) {
        const double wgt = std::exp(-(d2 * d2) / (2.0 * sigma * sigma));
        ws += wgt;
        q0s[0] += wgt * R.q0[2 * id];
        q0s[1] += wgt * R.q0[2 * id + 1];
        nb.push_back(id);
        tm += R.m0[id];
        tv += R.vol0[id];
      }
    });
    const int count = (int)nb.size();
    // with no neighbour the reference leaves 0/0 here
    R.q0[2 * i] = q0s[0] / ws;
    R.q0[2 * i + 1] = q0s[1] / ws;
    R.m0[i] = tm / (count + 1.0);
    R.vol0[i] = tv / (count + 1.0);
    const double factor = (double)count / (double)(count + 1.0);
    for (int id : nb) {
      R.m0[id] *= factor;
      R.vol0[id] *= factor;
    }
  }
  const double h1 = R.hl.empty() ? 0.0 : R.hl[0];
  // node fields to each inserted point, independently: over host threads
  hg::host_parallel((size_t)(after - before), 256, [&](size_t pb, size_t pe) {
  for (int64_t p = before + (int64_t)pb; p < before + (int64_t)pe; ++p) {
    const double x = R.q[2 * p], y = R.q[2 * p + 1];
    double Jv[1], be[4], vel[2];
    interp_nodes(R, x, y, h1, zd.mpm_grid_min[0], zd.mpm_grid_min[1], R.grid_h, zd.mpm_cells[0],
                 fJ, 1, Jv);
    interp_nodes(R, x, y, h1, zd.mpm_grid_min[0], zd.mpm_grid_min[1], R.grid_h, zd.mpm_cells[0],
                 fb, 4, be);
    const double sd = std::sqrt(det2(be));
    for (int c = 0; c < 4; ++c) be[c] /= sd;
    interp_nodes(R, x, y, h1, zd.mpm_grid_min[0], zd.mpm_grid_min[1], R.grid_h, zd.mpm_cells[0],
                 fv, 2, vel);
    R.v[2 * p] = vel[0];
    R.v[2 * p + 1] = vel[1];
    if (R.d.newly_inserted_continuum_stress_free) {
      R.J[p] = 1.0;
      be[0] = 1.0, be[1] = 0.0, be[2] = 0.0, be[3] = 1.0;
    } else {
      R.J[p] = Jv[0];
    }
    for (int c = 0; c < 4; ++c) R.be[4 * p + c] = be[c];
  }
  });
}

template <typename T> void compact(std::vector<T> &a, const std::vector<uint8_t> &keep, int width) {
  size_t to = 0;
  for (size_t i = 0; i < keep.size(); ++i) {
    if (!keep[i]) continue;
    if (to != i)
      for (int c = 0; c < width; ++c) a[to * width + c] = a[i * width + c];
    ++to;
  }
  a.resize(to * width);
}

// deleteParticlesUsingZoneIndicators (ResamplingTools.cpp:28-56) with
// MaterialPoints::deleteMaterialPoint and RigidBody2DState::removeBodies.
void delete_by_zone(hg_resampler &R, const hg_zones &z) {
  // labels over host threads; each array compacted as one task of the pool
  // (every array keeps the same elements in the same order)
  const size_t n = npoints(R);
  std::vector<uint8_t> keep(n, 1);
  hg::host_parallel(n, 8192, [&](size_t b, size_t e) {
    for (size_t p = b; p < e; ++p) {
      const int32_t l = hg::zone_label_at(z, R.q[2 * p], R.q[2 * p + 1]);
      if (l < 0 || l == HG_ZONE_DISCRETE) keep[p] = 0;
    }
  });
  R.stats.points_deleted += (int64_t)std::count(keep.begin(), keep.end(), 0);
  const size_t nb = nbodies(R);
  std::vector<uint8_t> keepb(nb, 1);
  hg::host_parallel(nb, 8192, [&](size_t b0, size_t b1) {
    for (size_t b = b0; b < b1; ++b) {
      if (R.fixed[b]) continue;
      const int32_t l = hg::zone_label_at(z, R.dq[3 * b], R.dq[3 * b + 1]);
      if (l < 0 || l == HG_ZONE_CONTINUUM) keepb[b] = 0;
    }
  });
  R.dem_map.assign(nb, -1);
  int32_t next = 0;
  for (size_t b = 0; b < nb; ++b)
    if (keepb[b]) R.dem_map[b] = next++;
  R.stats.grains_deleted += (int64_t)(nb - (size_t)next);
  const std::function<void()> tasks[] = {
      [&] { compact(R.q0, keep, 2); },    [&] { compact(R.q, keep, 2); },
      [&] { compact(R.v, keep, 2); },     [&] { compact(R.m, keep, 1); },
      [&] { compact(R.vol, keep, 1); },   [&] { compact(R.m0, keep, 1); },
      [&] { compact(R.vol0, keep, 1); },  [&] { compact(R.w, keep, 1); },
      [&] { compact(R.hl, keep, 1); },    [&] { compact(R.be, keep, 4); },
      [&] { compact(R.J, keep, 1); },     [&] { compact(R.jh, keep, 1); },
      [&] { compact(R.kin, keep, 1); },   [&] { compact(R.dq0, keepb, 3); },
      [&] { compact(R.dq, keepb, 3); },   [&] { compact(R.dv, keepb, 3); },
      [&] { compact(R.dr, keepb, 1); },   [&] { compact(R.M0, keepb, 3); },
      [&] { compact(R.dw, keepb, 1); },   [&] { compact(R.fixed, keepb, 1); }};
  hg::host_pool_run(sizeof(tasks) / sizeof(tasks[0]), [&](size_t k) { tasks[k](); });
}

// demWeight / mpmWeight with updateMassWeights / updateWeights
// (HybridGrains2DSim.cpp:512-528), over host threads
void update_weights(hg_resampler &R, const hg_zones &z) {
  hg::host_parallel(nbodies(R), 8192, [&](size_t b0, size_t b1) {
    for (size_t b = b0; b < b1; ++b) {
      const int32_t l = hg::zone_label_at(z, R.dq[3 * b], R.dq[3 * b + 1]);
      R.dw[b] = l == HG_ZONE_HYBRID ? 0.5 : (l == HG_ZONE_DISCRETE ? 1.0 : 0.0);
    }
  });
  hg::host_parallel(npoints(R), 8192, [&](size_t b, size_t e) {
    for (size_t p = b; p < e; ++p) {
      const int32_t l = hg::zone_label_at(z, R.q[2 * p], R.q[2 * p + 1]);
      R.w[p] = l == HG_ZONE_HYBRID ? 0.5 : (l == HG_ZONE_CONTINUUM ? 1.0 : 0.0);
      R.m[p] = R.m0[p] * R.w[p];
      R.vol[p] = R.vol0[p] * R.w[p];
    }
  });
}

double ms_since(std::chrono::steady_clock::time_point &t) {
  const auto now = std::chrono::steady_clock::now();
  const double ms = std::chrono::duration<double, std::milli>(now - t).count();
  t = now;
  return ms;
}

hg_status run(hg_resampler &R, const hg_zones &z) {
  R.stats = hg_resampler_stats{};
  auto t = std::chrono::steady_clock::now();
  const bool direct = z.d.allow_direct_transitions != 0;
  int64_t g_before = 0, p_before = 0, p_after = 0, p_mid = 0, dummy = 0;
  std::vector<Box> inner;
  hg::zone_inner_continuum(z, direct, inner);
  // The insertions draw their trial positions from R.mt in this order: the
  // grains over the hybrid zone, then the points over the hybrid zone, the
  // direct transitions and the inner continuum (two words per trial, 16
  // trials per region). The words are drawn here in that order; the grain
  // insertion (grains only, radii from its own engine) then runs on a
  // second host thread beside the point insertions (points only). The
  // mailbox stamp advances by all their tests at the end.
  const size_t Tg = 16 * z.rzones.size(), Tp1 = 16 * z.rzones.size();
  const size_t Tp2 = direct ? 16 * z.direct.size() : 0, Tp3 = 16 * inner.size();
  // (the grains' words first, so that their insertion can start; the
  // points' words on a third thread while this one builds the points'
  // search grid)
  static thread_local std::vector<uint32_t> tl_words;
  std::vector<uint32_t> &words = tl_words;
  words.resize(2 * (Tg + Tp1 + Tp2 + Tp3));
  R.mt.fill_raw(words.data(), 2 * Tg);
  const uint32_t *wg = words.data(), *wp1 = wg + 2 * Tg, *wp2 = wp1 + 2 * Tp1,
                 *wp3 = wp2 + 2 * Tp2;
  hg_status gst = HG_OK;
  double g_ms = 0.0;
  std::thread grains([&] {
    auto tg = std::chrono::steady_clock::now();
    gst = insert_grains(R, z.rzones, g_before, wg);
    g_ms = ms_since(tg);
  });
  std::thread point_words(
      [&] { R.mt.fill_raw(words.data() + 2 * Tg, words.size() - 2 * Tg); });
  hg_status st = HG_OK;
  // one search grid over the points for the three insertions, over the
  // extent of all their regions
  static thread_local FillGrid tl_pgrid;
  {
    const double rp = 0.5 * R.d.initial_particle_size;
    double e[4] = {0.0, 0.0, 0.0, 0.0};
    bool any = false;
    const std::vector<Box> *all[3] = {&z.rzones, &z.direct, &inner};
    for (const std::vector<Box> *regs : all) {
      if (regs->empty() || (regs == &z.direct && !direct)) continue;
      double f[4];
      regions_extent(*regs, rp, f);
      if (!any) std::copy(f, f + 4, e);
      e[0] = std::min(e[0], f[0]);
      e[1] = std::min(e[1], f[1]);
      e[2] = std::max(e[2], f[2]);
      e[3] = std::max(e[3], f[3]);
      any = true;
    }
    if (any) {
      const size_t n = npoints(R);
      std::vector<double> px(n), py(n), rad(n, rp);
      for (size_t p = 0; p < n; ++p) {
        px[p] = R.q[2 * p];
        py[p] = R.q[2 * p + 1];
      }
      build_fill_grid(tl_pgrid, e[0], e[1], e[2], e[3], rp, px, py, rad);
    }
  }
  point_words.join();
  int64_t i_before = 0, i_after = 0;
  st = insert_points(R, z.rzones, p_before, tl_pgrid, wp1);
  p_mid = (int64_t)npoints(R);
  if (st == HG_OK && direct) st = insert_points(R, z.direct, dummy, tl_pgrid, wp2);
  p_after = (int64_t)npoints(R);
  i_before = i_after = p_after;
  if (st == HG_OK && !inner.empty()) {
    st = insert_points(R, inner, i_before, tl_pgrid, wp3);
    i_after = (int64_t)npoints(R);
  }
  grains.join();
  if (gst != HG_OK) return gst;
  if (st != HG_OK) return st;
  advance_test_id(R.test_id, Tg + Tp1 + Tp2 + Tp3);
  const int64_t g_after = (int64_t)nbodies(R);
  // (the grain insertion's own time; the point insertions' wall time, with
  // the grain insertion beside them)
  R.stats.ms_insert_grains = g_ms;
  R.stats.ms_insert_points = ms_since(t);
  CellLists cont, disc;
  point_grids(R, cont, disc);
  R.stats.ms_point_grids = ms_since(t);
  if (direct) {
    hybrid_point_quantities(R, z.rzones, p_before, p_mid, g_before, cont, disc);
    hybrid_point_quantities(R, z.direct, p_mid, p_after, g_before, cont, disc);
  } else {
    hybrid_point_quantities(R, z.rzones, p_before, p_after, g_before, cont, disc);
  }
  grain_quantities(R, g_before, g_after, p_before, cont, disc);
  inner_point_quantities(R, i_before, i_after, cont);
  R.stats.ms_quantities = ms_since(t);
  delete_by_zone(R, z);
  update_weights(R, z);
  R.stats.ms_delete = ms_since(t);
  return HG_OK;
}

} // namespace

using hg::fail;

extern "C" {

hg_status hg_resampler_create(const hg_resampler_desc *d, hg_resampler **out) {
  if (!d || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (!(d->initial_particle_size > 0.0) || d->zones.mpm_cells[0] <= 0 || d->zones.mpm_cells[1] <= 0 ||
      !(d->zones.mpm_cell_width > 0.0) || !(d->mpm_grid_max[0] > d->zones.mpm_grid_min[0]))
    return fail(HG_ERR_INVALID_ARGUMENT, "invalid resampler description");
  if (d->basis != HG_BASIS_LINEAR && d->basis != HG_BASIS_UGIMP)
    return fail(HG_ERR_INVALID_ARGUMENT, "unknown basis");
  hg_resampler *r = new (std::nothrow) hg_resampler();
  if (!r) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  r->d = *d;
  // Grid::computeCellWidth (Grid.cpp:5-10): (max - min) / count along x
  r->grid_h = (d->mpm_grid_max[0] - d->zones.mpm_grid_min[0]) / (double)d->zones.mpm_cells[0];
  r->radius_dist = std::normal_distribution<double>(d->dem_r_mean, d->dem_r_std);
  *out = r;
  return HG_OK;
}

namespace {

// RNG blob: magic, MT19937 position and words, next test id, then the text
// forms (operator<<) of the radius engine and distribution, each length-
// prefixed.
constexpr char RNG_MAGIC[8] = {'H', 'G', 'R', 'N', 'G', '\0', '\0', '\1'};

std::string rng_text(const hg_resampler *r, int which) {
  std::ostringstream o;
  if (which == 0) o << r->gen;
  else o << r->radius_dist;
  return o.str();
}

int64_t rng_size(const hg_resampler *r) {
  return 8 + 4 + 4 * Mt19937::N + 4 + 8 + (int64_t)rng_text(r, 0).size() + 8 +
         (int64_t)rng_text(r, 1).size();
}

} // namespace

hg_status hg_resampler_rng_bytes(hg_resampler *r, int64_t *bytes) {
  if (!r || !bytes) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *bytes = rng_size(r);
  return HG_OK;
}

hg_status hg_resampler_rng_save(hg_resampler *r, void *dst, int64_t bytes) {
  if (!r || !dst) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (bytes < rng_size(r)) return fail(HG_ERR_CAPACITY, "RNG buffer too small");
  unsigned char *o = static_cast<unsigned char *>(dst);
  auto put = [&](const void *p, size_t n) {
    std::memcpy(o, p, n);
    o += n;
  };
  put(RNG_MAGIC, 8);
  const int32_t pos = r->mt.i, tid = r->test_id;
  put(&pos, 4);
  put(r->mt.s, 4 * Mt19937::N);
  put(&tid, 4);
  for (int w = 0; w < 2; ++w) {
    const std::string t = rng_text(r, w);
    const int64_t len = (int64_t)t.size();
    put(&len, 8);
    put(t.data(), t.size());
  }
  return HG_OK;
}

hg_status hg_resampler_rng_load(hg_resampler *r, const void *src, int64_t bytes) {
  if (!r || !src) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  const unsigned char *p = static_cast<const unsigned char *>(src), *end = p + bytes;
  auto get = [&](void *d, size_t n) {
    if (p + n > end) return false;
    std::memcpy(d, p, n);
    p += n;
    return true;
  };
  char magic[8];
  int32_t pos = 0, tid = 0;
  Mt19937 mt;
  if (!get(magic, 8) || std::memcmp(magic, RNG_MAGIC, 8) != 0 || !get(&pos, 4) ||
      !get(mt.s, 4 * Mt19937::N) || !get(&tid, 4) || pos < 0 || pos > Mt19937::N + 1)
    return fail(HG_ERR_INVALID_ARGUMENT, "not a resampler RNG blob");
  std::string text[2];
  for (int w = 0; w < 2; ++w) {
    int64_t len = 0;
    if (!get(&len, 8) || len < 0 || p + len > end)
      return fail(HG_ERR_INVALID_ARGUMENT, "truncated resampler RNG blob");
    text[w].assign(reinterpret_cast<const char *>(p), (size_t)len);
    p += len;
  }
  std::default_random_engine gen;
  std::normal_distribution<double> dist;
  std::istringstream a(text[0]), b(text[1]);
  a >> gen;
  b >> dist;
  if (a.fail() || b.fail()) return fail(HG_ERR_INVALID_ARGUMENT, "malformed resampler RNG blob");
  mt.i = pos;
  r->mt = mt;
  r->gen = gen;
  r->radius_dist = dist;
  r->test_id = tid;
  return HG_OK;
}

hg_status hg_resampler_destroy(hg_resampler *r) {
  delete r;
  return HG_OK;
}

hg_status hg_resampler_set_points(hg_resampler *r, int64_t n, const double *q0, const double *q,
                                  const double *v, const double *m, const double *vol,
                                  const double *m0, const double *vol0, const double *hl,
                                  const double *be, const double *J, const int32_t *jh,
                                  const uint8_t *kin) {
  if (!r || n < 0) return fail(HG_ERR_INVALID_ARGUMENT, "invalid argument");
  if (n > 0 && (!q0 || !q || !v || !m || !vol || !m0 || !vol0 || !hl || !be || !J))
    return fail(HG_ERR_INVALID_ARGUMENT, "NULL array");
  const size_t k = (size_t)n;
  // one array per task of the host pool
  const std::function<void()> tasks[] = {
      [&] { r->q0.assign(q0, q0 + 2 * k); },   [&] { r->q.assign(q, q + 2 * k); },
      [&] { r->v.assign(v, v + 2 * k); },      [&] { r->m.assign(m, m + k); },
      [&] { r->vol.assign(vol, vol + k); },    [&] { r->m0.assign(m0, m0 + k); },
      [&] { r->vol0.assign(vol0, vol0 + k); }, [&] { r->w.assign(k, 1.0); },
      [&] { r->hl.assign(hl, hl + k); },       [&] { r->be.assign(be, be + 4 * k); },
      [&] { r->J.assign(J, J + k); },
      [&] {
        if (jh) r->jh.assign(jh, jh + k);
        else r->jh.assign(k, 0);
      },
      [&] {
        if (kin) r->kin.assign(kin, kin + k);
        else r->kin.assign(k, 0);
      }};
  hg::host_pool_run(sizeof(tasks) / sizeof(tasks[0]), [&](size_t t) { tasks[t](); });
  return HG_OK;
}

hg_status hg_resampler_set_grains(hg_resampler *r, int64_t n, const double *q0, const double *q,
                                  const double *v, const double *radius, const double *M0,
                                  const uint8_t *fixed) {
  if (!r || n < 0) return fail(HG_ERR_INVALID_ARGUMENT, "invalid argument");
  if (n > 0 && (!q0 || !q || !v || !radius || !M0)) return fail(HG_ERR_INVALID_ARGUMENT, "NULL array");
  const size_t k = (size_t)n;
  r->dq0.assign(q0, q0 + 3 * k);
  r->dq.assign(q, q + 3 * k);
  r->dv.assign(v, v + 3 * k);
  r->dr.assign(radius, radius + k);
  r->M0.assign(M0, M0 + 3 * k);
  r->dw.assign(k, 1.0);
  if (fixed) r->fixed.assign(fixed, fixed + k);
  else r->fixed.assign(k, 0);
  r->dem_map.clear();
  return HG_OK;
}

hg_status hg_resampler_set_homogenized(hg_resampler *r, const double *stress, const double *velocity) {
  if (!r) return fail(HG_ERR_INVALID_ARGUMENT, "r is NULL");
  const size_t nn = (size_t)(r->d.zones.mpm_cells[0] + 1) * (r->d.zones.mpm_cells[1] + 1);
  hg::host_pool_run(2, [&](size_t t) {
    if (t == 0) {
      if (stress) r->hs.assign(stress, stress + 4 * nn);
      else r->hs.assign(4 * nn, 0.0);
    } else {
      if (velocity) r->hv.assign(velocity, velocity + 2 * nn);
      else r->hv.assign(2 * nn, 0.0);
    }
  });
  return HG_OK;
}

hg_status hg_resampler_run(hg_resampler *r, hg_zones *z) {
  HG_TRACE("hg_resampler_run");
  if (!r || !z) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  const hg_zones_desc &a = r->d.zones, &b = z->d;
  if (a.mpm_cells[0] != b.mpm_cells[0] || a.mpm_cells[1] != b.mpm_cells[1] ||
      a.mpm_cell_width != b.mpm_cell_width || a.mpm_grid_min[0] != b.mpm_grid_min[0] ||
      a.mpm_grid_min[1] != b.mpm_grid_min[1])
    return fail(HG_ERR_INVALID_ARGUMENT, "zone labels of another grid");
  if ((r->d.homogenize_stress || r->d.homogenize_velocity) && r->hs.empty())
    hg_resampler_set_homogenized(r, nullptr, nullptr);
  return run(*r, *z);
}

hg_status hg_resampler_counts(hg_resampler *r, int64_t *points, int64_t *grains,
                              hg_resampler_stats *stats) {
  if (!r) return fail(HG_ERR_INVALID_ARGUMENT, "r is NULL");
  if (points) *points = (int64_t)npoints(*r);
  if (grains) *grains = (int64_t)nbodies(*r);
  if (stats) *stats = r->stats;
  return HG_OK;
}

hg_status hg_resampler_get_points(hg_resampler *r, double *q0, double *q, double *v, double *m,
                                  double *vol, double *m0, double *vol0, double *w, double *hl,
                                  double *be, double *J, int32_t *jh, uint8_t *kin) {
  if (!r) return fail(HG_ERR_INVALID_ARGUMENT, "r is NULL");
  auto put = [](const auto &src, auto *dst) {
    if (dst) std::copy(src.begin(), src.end(), dst);
  };
  // one array per task of the host pool
  const std::function<void()> tasks[] = {
      [&] { put(r->q0, q0); },     [&] { put(r->q, q); },   [&] { put(r->v, v); },
      [&] { put(r->m, m); },       [&] { put(r->vol, vol); }, [&] { put(r->m0, m0); },
      [&] { put(r->vol0, vol0); }, [&] { put(r->w, w); },   [&] { put(r->hl, hl); },
      [&] { put(r->be, be); },     [&] { put(r->J, J); },   [&] { put(r->jh, jh); },
      [&] { put(r->kin, kin); }};
  hg::host_pool_run(sizeof(tasks) / sizeof(tasks[0]), [&](size_t t) { tasks[t](); });
  return HG_OK;
}

hg_status hg_resampler_get_grains(hg_resampler *r, double *q0, double *q, double *v, double *radius,
                                  double *M0, double *w, uint8_t *fixed, int32_t *old_to_new) {
  if (!r) return fail(HG_ERR_INVALID_ARGUMENT, "r is NULL");
  auto put = [](const auto &src, auto *dst) {
    if (dst) std::copy(src.begin(), src.end(), dst);
  };
  put(r->dq0, q0);
  put(r->dq, q);
  put(r->dv, v);
  put(r->dr, radius);
  put(r->M0, M0);
  put(r->dw, w);
  put(r->fixed, fixed);
  put(r->dem_map, old_to_new);
  return HG_OK;
}

hg_status hg_resampler_dem_map_size(hg_resampler *r, int64_t *n) {
  if (!r || !n) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = (int64_t)r->dem_map.size();
  return HG_OK;
}

uint32_t hg_resampler_random_u32(hg_resampler *r) { return r ? r->mt.next() : 0u; }
float hg_resampler_random_f32(hg_resampler *r) { return r ? r->mt.uniform() : 0.0f; }
double hg_resampler_random_radius(hg_resampler *r) { return r ? r->radius_dist(r->gen) : 0.0; }

} // extern "C"
