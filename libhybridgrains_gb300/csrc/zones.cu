// Zone labels of the hybrid method (ZoneTools, hybridgrains2dnew/ZoneTools.
// cpp:6-758), host code run at the resampling interval on positions copied
// from the device.
//
// Per update:
//   1. packing fraction on the level-set grid: per cell, the mean over
//      S x S sample windows of (area of the disks inside the window) /
//      (window area); cells near material points are set to 1
//      (updatePackingFraction, ZoneTools.cpp:186-276);
//   2. a distance field from points sampled on the cell edges where the
//      packing fraction crosses the threshold, propagated to the grid
//      points by a breadth-first sweep, signed positive around dense cells
//      (updateDistanceField, ZoneTools.cpp:289-445; redistanceGrid,
//      levelsetutil.cpp:27-144);
//   3. labels: level-set cells by the distance range at their corners, then
//      MPM cells from the level-set cells they overlap with the hysteresis of
//      the previous labels (computeRZones, ZoneTools.cpp:447-672).
//
// The labels are compared with thresholds, so they are computed here with
// the reference's FP64 expressions in its order (this file is compiled
// without FMA contraction); they are bit-exact against the oracle.
//
// Layout: the disk lists per level-set cell are one CSR array (counting sort
// in disk order, the order the reference's per-cell lists have), and rows of
// the packing-fraction grid are computed by worker threads (each cell's sum
// is independent of the others, so the result does not depend on them).
#include "hg_internal.cuh"
#include "zones_internal.cuh"

#include <algorithm>
#include <cmath>
#include <new>
#include <thread>
#include <vector>

namespace {

// Area of the intersection of the disk (cx, cy, r) with the box
// [x0, x1] x [y0, y1] (published construction: integrate the circle segment
// over vertical strips of the box, splitting the box at the centre's y).
double chord_half(double h, double r) { return h < r ? std::sqrt(r * r - h * h) : 0.0; }

double segment_integral(double x, double h, double r) {
  return 0.5 * (std::sqrt(1.0 - x * x / (r * r)) * x * r + r * r * std::asin(x / r) - 2.0 * h * x);
}

// The part of the disk above y = h and between x0 and x1 (centre at 0).
double strip_area(double x0, double x1, double h, double r) {
  if (x0 > x1) std::swap(x0, x1);
  const double s = chord_half(h, r);
  return segment_integral(std::max(-s, std::min(s, x1)), h, r) -
         segment_integral(std::max(-s, std::min(s, x0)), h, r);
}

double box_area(double x0, double x1, double y0, double y1, double r) {
  if (y0 > y1) std::swap(y0, y1);
  if (y0 < 0.0) {
    if (y1 < 0.0) return box_area(x0, x1, -y0, -y1, r);
    return box_area(x0, x1, 0.0, -y0, r) + box_area(x0, x1, 0.0, y1, r);
  }
  return strip_area(x0, x1, y0, r) - strip_area(x0, x1, y1, r);
}

double disk_box_area(double x0, double x1, double y0, double y1, double cx, double cy, double r) {
  return box_area(x0 - cx, x1 - cx, y0 - cy, y1 - cy, r);
}

} // namespace


namespace {

constexpr int32_t ZC = HG_ZONE_CONTINUUM, ZD = HG_ZONE_DISCRETE, ZH = HG_ZONE_HYBRID;

// CUniformGridH2D::getGridID: clamped floor of the grid coordinate.
inline void grid_id(const hg_zones &z, double x, double y, unsigned &i, unsigned &j) {
  const double u = (x - z.ls_min[0]) / z.ls_h, v = (y - z.ls_min[1]) / z.ls_h;
  i = (unsigned)std::max<int>(0, std::min<int>((int)z.N[0] - 1, (int)std::floor(u)));
  j = (unsigned)std::max<int>(0, std::min<int>((int)z.N[1] - 1, (int)std::floor(v)));
}

void packing_fraction(hg_zones &z, int64_t nd, const double *q3, const double *r,
                      const uint8_t *fixed, int64_t np, const double *pq) {
  const unsigned nx = z.N[0], ny = z.N[1];
  const double w = z.d.phi_window_size;
  const int S = z.d.phi_samples_per_cell_side;
  std::fill(z.phi.begin(), z.phi.end(), 0.0);
  // non-fixed disks in body order (getAllNonFixedCircleBodies)
  std::vector<double> px, py, pr;
  for (int64_t b = 0; b < nd; ++b) {
    if (fixed && fixed[b]) continue;
    px.push_back(q3[3 * b]);
    py.push_back(q3[3 * b + 1]);
    pr.push_back(r[b]);
  }
  const int64_t n = (int64_t)px.size();
  // CSR of disks per cell of their clamped box range, in disk order
  std::vector<unsigned> lo(2 * n), hi(2 * n);
  std::vector<int64_t> start((size_t)nx * ny + 1, 0);
  for (int64_t k = 0; k < n; ++k) {
    grid_id(z, px[k] - pr[k], py[k] - pr[k], lo[2 * k], lo[2 * k + 1]);
    grid_id(z, px[k] + pr[k], py[k] + pr[k], hi[2 * k], hi[2 * k + 1]);
    for (unsigned j = lo[2 * k + 1]; j <= hi[2 * k + 1]; ++j)
      for (unsigned i = lo[2 * k]; i <= hi[2 * k]; ++i) start[(size_t)j * nx + i + 1]++;
  }
  for (size_t c = 0; c < (size_t)nx * ny; ++c) start[c + 1] += start[c];
  std::vector<int32_t> ids(start.back());
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t k = 0; k < n; ++k)
      for (unsigned j = lo[2 * k + 1]; j <= hi[2 * k + 1]; ++j)
        for (unsigned i = lo[2 * k]; i <= hi[2 * k]; ++i)
          ids[fill[(size_t)j * nx + i]++] = (int32_t)k;
  }
  // One window: each disk counts once, at the first cell of the window's
  // cell range (row-major) where it is listed.
  auto window = [&](double x0, double y0, double x1, double y1) {
    const double area = (x1 - x0) * (y1 - y0);
    unsigned i0, j0, i1, j1;
    grid_id(z, x0, y0, i0, j0);
    grid_id(z, x1, y1, i1, j1);
    double tot = 0.0;
    for (unsigned j = j0; j <= j1; ++j)
      for (unsigned i = i0; i <= i1; ++i) {
        const size_t c = (size_t)j * nx + i;
        for (int64_t e = start[c]; e < start[c + 1]; ++e) {
          const int32_t k = ids[e];
          const unsigned fi = std::max(i0, lo[2 * k]), fj = std::max(j0, lo[2 * k + 1]);
          if (fi != i || fj != j) continue; // seen at an earlier cell
          tot += disk_box_area(x0, x1, y0, y1, px[k], py[k], pr[k]);
        }
      }
    return tot / area;
  };
  auto rows = [&](unsigned jb, unsigned je) {
    for (unsigned j = jb; j < je; ++j)
      for (unsigned i = 0; i < nx; ++i) {
        double pf = 0.0;
        for (int v = 0; v < S; ++v)
          for (int u = 0; u < S; ++u) {
            const double cx = z.ls_min[0] + ((double)i + ((double)u + 0.5) / S) * z.ls_h;
            const double cy = z.ls_min[1] + ((double)j + ((double)v + 0.5) / S) * z.ls_h;
            pf += window(cx - w * 0.5, cy - w * 0.5, cx + w * 0.5, cy + w * 0.5);
          }
        z.phi[(size_t)j * nx + i] = pf / (double)(S * S);
      }
  };
  // (rows taken in turn by the host threads: the disks fill a band of them)
  hg::host_parallel_dynamic(ny, 2, [&](size_t jb, size_t je) { rows((unsigned)jb, (unsigned)je); });
  // cells within half a window of a material point count as dense; the
  // reference's test excludes the first row and column (gid > 0)
  // (marks over host threads by points, each a relaxed atomic store of the
  // same value; then the marked cells' fractions set to 1)
  static thread_local std::vector<uint8_t> tl_mark;
  std::vector<uint8_t> &mark = tl_mark;
  mark.assign((size_t)nx * ny, 0);
  hg::host_parallel((size_t)np, 8192, [&](size_t pb, size_t pe) {
    for (size_t p = pb; p < pe; ++p) {
      const double x = pq[2 * p] - z.ls_min[0], y = pq[2 * p + 1] - z.ls_min[1];
      const int gj0 = (int)std::floor((y - w * 0.5) / z.ls_h);
      const int gj1 = (int)std::floor((y + w * 0.5) / z.ls_h);
      const int j0 = std::max(gj0, 1), j1 = std::min(gj1, (int)ny - 1);
      if (j0 > j1) continue;
      const int gi0 = (int)std::floor((x - w * 0.5) / z.ls_h);
      const int gi1 = (int)std::floor((x + w * 0.5) / z.ls_h);
      for (int j = j0; j <= j1; ++j)
        for (int i = std::max(gi0, 1); i <= std::min(gi1, (int)nx - 1); ++i)
          __atomic_store_n(&mark[(size_t)j * nx + i], (uint8_t)1, __ATOMIC_RELAXED);
    }
  });
  hg::host_parallel((size_t)nx * ny, 16384, [&](size_t cb, size_t ce) {
    for (size_t c = cb; c < ce; ++c)
      if (mark[c]) z.phi[c] = 1.0;
  });
}

void distance_field(hg_zones &z) {
  const unsigned nx = z.N[0], ny = z.N[1];
  const double thr = z.d.phi_threshold, h = z.ls_h;
  const auto dense = [&](unsigned i, unsigned j) { return z.phi[(size_t)j * nx + i] > thr; };
  std::vector<double> sx, sy;
  auto edge = [&](double ax, double ay, double bx, double by) {
    for (int k = 0; k < 4; ++k) {
      const double s = (k + 0.5) / 4;
      sx.push_back((1.0 - s) * ax + s * bx);
      sy.push_back((1.0 - s) * ay + s * by);
    }
  };
  // horizontal edges, placed at the top of row j (the reference's placement)
  for (unsigned j = 0; j <= ny; ++j)
    for (unsigned i = 0; i < nx; ++i) {
      const double cl = z.ls_min[0] + i * h, cr = z.ls_min[0] + (i + 1) * h;
      const double ct = z.ls_min[1] + (j + 1) * h;
      bool cross;
      if (j == 0) cross = dense(i, 0);
      else if (j == ny) cross = dense(i, ny - 1);
      else cross = dense(i, j - 1) != dense(i, j);
      if (cross) edge(cl, ct, cr, ct);
    }
  for (unsigned j = 0; j < ny; ++j)
    for (unsigned i = 0; i <= nx; ++i) {
      const double cl = z.ls_min[0] + i * h;
      const double cb = z.ls_min[1] + j * h, ct = z.ls_min[1] + (j + 1) * h;
      bool cross;
      if (i == 0) cross = dense(0, j);
      else if (i == nx) cross = dense(nx - 1, j);
      else cross = dense(i - 1, j) != dense(i, j);
      if (cross) edge(cl, cb, cl, ct);
    }
  z.n_boundary_samples = (int64_t)sx.size();
  // nearest sample per grid point: seed within 3h of every sample, then
  // propagate to the four neighbours breadth first
  const size_t npts = (size_t)(nx + 1) * (ny + 1);
  // distance and sample per grid point side by side (one line per visit)
  struct Nearest {
    double d;
    int64_t sample; // -1: none yet
  };
  std::vector<Nearest> near(npts, Nearest{1.0e10, -1});
  const double W = z.ls_max[0] - z.ls_min[0], H = z.ls_max[1] - z.ls_min[1];
  auto gpx = [&](int i) { return W * (double)i / (double)nx + z.ls_min[0]; };
  auto gpy = [&](int j) { return H * (double)j / (double)ny + z.ls_min[1]; };
  auto norm = [](double a, double b) { return std::sqrt(a * a + b * b); };
  // (over host threads by bands of grid rows: every grid point still sees
  // the samples in order, so ties go to the same sample)
  hg::host_parallel((size_t)ny + 1, 16, [&](size_t rb, size_t re) {
    for (size_t p = 0; p < sx.size(); ++p) {
      const double r = 3.0 * h;
      const double x0 = sx[p] - r, y0 = sy[p] - r, x1 = sx[p] + r, y1 = sy[p] + r;
      auto lo = [&](double v, double m, double ext, unsigned n) {
        return std::max<int>(0, std::min<int>((int)n, (int)std::floor((double)n * (v - m) / ext)));
      };
      auto up = [&](double v, double m, double ext, unsigned n) {
        return std::max<int>(0, std::min<int>((int)n, (int)std::ceil((double)n * (v - m) / ext)));
      };
      const int j0 = std::max(lo(y0, z.ls_min[1], H, ny), (int)rb);
      const int j1 = std::min(up(y1, z.ls_min[1], H, ny), (int)re - 1);
      if (j0 > j1) continue;
      const int i0 = lo(x0, z.ls_min[0], W, nx), i1 = up(x1, z.ls_min[0], W, nx);
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
          const size_t f = (size_t)j * (nx + 1) + i;
          const double dd = norm(gpx(i) - sx[p], gpy(j) - sy[p]);
          if (dd < near[f].d) {
            near[f].d = dd;
            near[f].sample = (int64_t)p;
          }
        }
    }
  });
  // (grid point coordinates tabulated with the same expressions; queue
  // entries carry their column and row)
  std::vector<double> tgx(nx + 1), tgy(ny + 1);
  for (unsigned i = 0; i <= nx; ++i) tgx[i] = gpx((int)i);
  for (unsigned j = 0; j <= ny; ++j) tgy[j] = gpy((int)j);
  std::vector<uint32_t> ring; // (column, row) pairs
  ring.reserve(2 * npts);
  for (size_t f = 0; f < npts; ++f)
    if (near[f].sample >= 0) {
      ring.push_back((uint32_t)(f % (nx + 1)));
      ring.push_back((uint32_t)(f / (nx + 1)));
    }
  for (size_t head = 0; head < ring.size(); head += 2) {
    const unsigned gi = ring[head], gj = ring[head + 1];
    const size_t f = (size_t)gj * (nx + 1) + gi;
    const int64_t cp = near[f].sample;
    const double spx = sx[cp], spy = sy[cp];
    auto visit = [&](unsigned ni, unsigned nj) {
      Nearest &g = near[(size_t)nj * (nx + 1) + ni];
      const double ex = tgx[ni] - spx, ey = tgy[nj] - spy, e2 = ex * ex + ey * ey;
      // a squared distance clearly above the stored one cannot win: the
      // square root (rounded to half an ulp) stays above it too
      if (g.sample >= 0 && e2 > g.d * g.d * (1.0 + 1.0e-12)) return;
      const double dd = norm(ex, ey);
      if (dd < g.d || g.sample < 0) {
        g.d = dd;
        g.sample = cp;
        ring.push_back(ni);
        ring.push_back(nj);
      }
    };
    // left, below, right, above
    if (gi > 0) visit(gi - 1, gj);
    if (gj > 0) visit(gi, gj - 1);
    if (gi < nx) visit(gi + 1, gj);
    if (gj < ny) visit(gi, gj + 1);
  }
  // sign: positive at the corners of dense cells
  std::vector<uint8_t> pos(npts, 0);
  for (unsigned j = 0; j < ny; ++j)
    for (unsigned i = 0; i < nx; ++i)
      if (dense(i, j)) {
        const size_t bl = (size_t)j * (nx + 1) + i, tl = bl + (nx + 1);
        pos[bl] = pos[bl + 1] = pos[tl] = pos[tl + 1] = 1;
      }
  for (size_t f = 0; f < npts; ++f) z.dist[f] = pos[f] ? std::fabs(near[f].d) : -std::fabs(near[f].d);
}

void labels(hg_zones &z) {
  const unsigned nx = z.N[0], ny = z.N[1];
  const double lvl = z.d.rzone_level_set, half = z.d.rzone_half_thickness;
  // Both passes over host threads in chunks of rows, each chunk listing its
  // boxes in (row, column) order; the lists join in chunk order, the order of
  // the sequential pass.
  constexpr unsigned ROWS = 8;
  auto chunked = [](unsigned rows, std::vector<hg_zones::Box> &out, auto body) {
    const size_t nc = (rows + ROWS - 1) / ROWS;
    std::vector<std::vector<hg_zones::Box>> part(nc);
    hg::host_parallel(nc, 2, [&](size_t cb, size_t ce) {
      for (size_t c = cb; c < ce; ++c)
        body((unsigned)(c * ROWS), std::min<unsigned>(rows, (unsigned)((c + 1) * ROWS)), part[c]);
    });
    for (auto &v : part) out.insert(out.end(), v.begin(), v.end());
  };
  z.ls_rzones.clear();
  chunked(ny, z.ls_rzones, [&](unsigned jb, unsigned je, std::vector<hg_zones::Box> &ls_rzones) {
  for (unsigned j = jb; j < je; ++j)
    for (unsigned i = 0; i < nx; ++i) {
      const size_t a = (size_t)j * (nx + 1) + i, b = a + (nx + 1);
      const double dmin = std::min(std::min(z.dist[a], z.dist[a + 1]), std::min(z.dist[b], z.dist[b + 1]));
      const double dmax = std::max(std::max(z.dist[a], z.dist[a + 1]), std::max(z.dist[b], z.dist[b + 1]));
      int32_t &lab = z.ls_label[(size_t)j * nx + i];
      if (dmax <= lvl - half) {
        lab = ZD;
      } else if (dmin >= lvl + half) {
        lab = ZC;
      } else {
        lab = ZH;
        const double ddx = (z.ls_max[0] - z.ls_min[0]) / (double)nx;
        const double ddy = (z.ls_max[1] - z.ls_min[1]) / (double)ny;
        hg_zones::Box bx{{z.ls_min[0] + ddx * (double)i, z.ls_min[1] + ddy * (double)j,
                          z.ls_min[0] + ddx * (i + 1.0), z.ls_min[1] + ddy * (j + 1.0)},
                         {(int32_t)i, (int32_t)j}};
        ls_rzones.push_back(bx);
      }
    }
  });
  // MPM cells from the level-set cells they overlap, with hysteresis
  z.prev = z.label;
  z.rzones.clear();
  z.direct.clear();
  const int mx = z.d.mpm_cells[0], my = z.d.mpm_cells[1];
  const double cw = z.d.mpm_cell_width;
  const bool direct_ok = z.d.allow_direct_transitions != 0;
  // the direct transitions of each chunk, joined after the pass
  const size_t nchunk = ((unsigned)my + ROWS - 1) / ROWS;
  std::vector<std::vector<hg_zones::Box>> direct_part(nchunk);
  chunked((unsigned)my, z.rzones, [&](unsigned jb, unsigned je, std::vector<hg_zones::Box> &rzones) {
  std::vector<hg_zones::Box> &direct = direct_part[jb / ROWS];
  for (int j = (int)jb; j < (int)je; ++j)
    for (int i = 0; i < mx; ++i) {
      const double x0 = z.d.mpm_grid_min[0] + (double)i * cw;
      const double y0 = z.d.mpm_grid_min[1] + (double)j * cw;
      const double x1 = z.d.mpm_grid_min[0] + ((double)i + 1.0) * cw;
      const double y1 = z.d.mpm_grid_min[1] + ((double)j + 1.0) * cw;
      auto clampi = [](int v, unsigned n) { return std::min<int>((int)n - 1, std::max<int>(0, v)); };
      const int u0 = clampi((int)std::floor((x0 - z.ls_min[0]) / z.ls_h), nx);
      const int v0 = clampi((int)std::floor((y0 - z.ls_min[1]) / z.ls_h), ny);
      const int u1 = clampi((int)std::floor((x1 - z.ls_min[0]) / z.ls_h), nx);
      const int v1 = clampi((int)std::floor((y1 - z.ls_min[1]) / z.ls_h), ny);
      int nh = 0, nc = 0, nd = 0;
      for (int v = v0; v <= v1; ++v)
        for (int u = u0; u <= u1; ++u) {
          const int32_t l = z.ls_label[(size_t)v * nx + u];
          nh += l == ZH;
          nc += l == ZC;
          nd += l == ZD;
        }
      const size_t f = (size_t)j * mx + i;
      const int32_t was = z.prev[f];
      const hg_zones::Box bx{{x0, y0, x1, y1}, {i, j}};
      int32_t lab = was; // kept when no level-set cell overlaps (cannot happen)
      if (nh > 0 || (nd > 0 && nc > 0)) {
        lab = ZH;
      } else if (nd > 0) {
        lab = (direct_ok || was == ZD || was == ZH) ? ZD : ZH;
      } else if (nc > 0) {
        if (direct_ok) {
          lab = ZC;
          if (was == ZD) direct.push_back(bx);
        } else {
          lab = (was == ZC || was == ZH) ? ZC : ZH;
        }
      }
      z.label[f] = lab;
      if (lab == ZH && nh + nc + nd > 0) rzones.push_back(bx);
    }
  });
  for (auto &v : direct_part) z.direct.insert(z.direct.end(), v.begin(), v.end());
}


} // namespace

using hg::fail;

extern "C" {

hg_status hg_zones_create(const hg_zones_desc *d, hg_zones **out) {
  if (!d || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (!(d->mpm_cell_width > 0.0) || !(d->level_set_cell_width > 0.0) || d->mpm_cells[0] <= 0 ||
      d->mpm_cells[1] <= 0 || d->phi_samples_per_cell_side <= 0 || !(d->phi_window_size > 0.0))
    return fail(HG_ERR_INVALID_ARGUMENT, "invalid zone description");
  // ZoneTools::init rejects a level-set cell wider than an MPM cell
  if (d->mpm_cell_width / d->level_set_cell_width < 1.0)
    return fail(HG_ERR_INVALID_ARGUMENT, "level-set cells must not be wider than MPM cells");
  hg_zones *z = new (std::nothrow) hg_zones();
  if (!z) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  z->d = *d;
  for (int a = 0; a < 2; ++a) {
    z->N[a] = (unsigned)std::ceil((double)d->mpm_cells[a] * d->mpm_cell_width / d->level_set_cell_width);
    z->ls_min[a] = d->mpm_grid_min[a];
    z->ls_max[a] = d->mpm_grid_min[a] + d->level_set_cell_width * (double)z->N[a];
  }
  z->ls_h = d->level_set_cell_width;
  const size_t cells = (size_t)z->N[0] * z->N[1];
  z->phi.assign(cells, 0.0);
  z->dist.assign((size_t)(z->N[0] + 1) * (z->N[1] + 1), 0.0);
  z->ls_label.assign(cells, ZD);
  z->label.assign((size_t)d->mpm_cells[0] * d->mpm_cells[1], ZD);
  z->prev = z->label;
  *out = z;
  return HG_OK;
}

hg_status hg_zones_destroy(hg_zones *z) {
  delete z;
  return HG_OK;
}

hg_status hg_zones_update(hg_zones *z, int64_t n_disks, const double *q, const double *radius,
                          const uint8_t *fixed, int64_t n_points, const double *points) {
  HG_TRACE("hg_zones_update");
  if (!z) return fail(HG_ERR_INVALID_ARGUMENT, "z is NULL");
  if (n_disks < 0 || n_points < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative count");
  if ((n_disks > 0 && (!q || !radius)) || (n_points > 0 && !points))
    return fail(HG_ERR_INVALID_ARGUMENT, "NULL array");
  packing_fraction(*z, n_disks, q, radius, fixed, n_points, points);
  distance_field(*z);
  labels(*z);
  return HG_OK;
}

hg_status hg_zones_grid_info(hg_zones *z, int32_t level_set_cells[2], int32_t mpm_cells[2]) {
  if (!z) return fail(HG_ERR_INVALID_ARGUMENT, "z is NULL");
  if (level_set_cells) {
    level_set_cells[0] = (int32_t)z->N[0];
    level_set_cells[1] = (int32_t)z->N[1];
  }
  if (mpm_cells) {
    mpm_cells[0] = z->d.mpm_cells[0];
    mpm_cells[1] = z->d.mpm_cells[1];
  }
  return HG_OK;
}

hg_status hg_zones_fields(hg_zones *z, double *packing_fraction_out, double *distance,
                          int32_t *level_set_labels, int32_t *mpm_labels) {
  if (!z) return fail(HG_ERR_INVALID_ARGUMENT, "z is NULL");
  if (packing_fraction_out) std::copy(z->phi.begin(), z->phi.end(), packing_fraction_out);
  if (distance) std::copy(z->dist.begin(), z->dist.end(), distance);
  if (level_set_labels) std::copy(z->ls_label.begin(), z->ls_label.end(), level_set_labels);
  if (mpm_labels) std::copy(z->label.begin(), z->label.end(), mpm_labels);
  return HG_OK;
}

hg_status hg_zones_set_labels(hg_zones *z, const int32_t *mpm_labels) {
  if (!z || !mpm_labels) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  std::copy(mpm_labels, mpm_labels + z->label.size(), z->label.begin());
  return HG_OK;
}

hg_status hg_zones_list(hg_zones *z, int32_t which, int64_t cap, double *boxes, int32_t *cells,
                        int64_t *count) {
  if (!z || !count) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  std::vector<hg_zones::Box> tmp;
  const std::vector<hg_zones::Box> *src = nullptr;
  switch (which) {
  case HG_ZONES_RECONCILIATION: src = &z->rzones; break;
  case HG_ZONES_DIRECT_TRANSITION: src = &z->direct; break;
  case HG_ZONES_LEVEL_SET_HYBRID: src = &z->ls_rzones; break;
  case HG_ZONES_INNER_CONTINUUM:
  case HG_ZONES_INNER_CONTINUUM_EXCLUDING_DIRECT:
    hg::zone_inner_continuum(*z, which == HG_ZONES_INNER_CONTINUUM_EXCLUDING_DIRECT, tmp);
    src = &tmp;
    break;
  default: return fail(HG_ERR_INVALID_ARGUMENT, "unknown zone list");
  }
  *count = (int64_t)src->size();
  const int64_t k = std::min<int64_t>(cap, *count);
  for (int64_t e = 0; e < k; ++e) {
    if (boxes)
      for (int c = 0; c < 4; ++c) boxes[4 * e + c] = (*src)[e].b[c];
    if (cells) {
      cells[2 * e] = (*src)[e].c[0];
      cells[2 * e + 1] = (*src)[e].c[1];
    }
  }
  return HG_OK;
}

hg_status hg_zones_to_delete(hg_zones *z, int32_t kind, int64_t n, const double *x,
                             int32_t stride, const uint8_t *fixed, int64_t cap, int32_t *ids,
                             int64_t *count) {
  if (!z || !count || (n > 0 && !x)) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (kind != HG_ZONES_MPM && kind != HG_ZONES_DEM) return fail(HG_ERR_INVALID_ARGUMENT, "unknown kind");
  if (stride < 2) return fail(HG_ERR_INVALID_ARGUMENT, "stride must be at least 2");
  // determineMPMParticlesToDelete / determineDEMGrainsToDelete: outside the
  // grid, or in the other method's full zone; fixed disks are kept
  const int32_t gone = kind == HG_ZONES_MPM ? ZD : ZC;
  int64_t c = 0;
  for (int64_t p = 0; p < n; ++p) {
    if (kind == HG_ZONES_DEM && fixed && fixed[p]) continue;
    const int32_t l = hg::zone_label_at(*z, x[(size_t)stride * p], x[(size_t)stride * p + 1]);
    if (l < 0 || l == gone) {
      if (ids && c < cap) ids[c] = (int32_t)p;
      ++c;
    }
  }
  *count = c;
  return HG_OK;
}

hg_status hg_zones_weights(hg_zones *z, int32_t kind, int64_t n, const double *x, int32_t stride,
                           double *w) {
  if (!z || (n > 0 && (!x || !w))) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (kind != HG_ZONES_MPM && kind != HG_ZONES_DEM) return fail(HG_ERR_INVALID_ARGUMENT, "unknown kind");
  if (stride < 2) return fail(HG_ERR_INVALID_ARGUMENT, "stride must be at least 2");
  // demWeight / mpmWeight (ZoneTools.cpp:123-147)
  const int32_t own = kind == HG_ZONES_MPM ? ZC : ZD;
  for (int64_t p = 0; p < n; ++p) {
    const int32_t l = hg::zone_label_at(*z, x[(size_t)stride * p], x[(size_t)stride * p + 1]);
    w[p] = l == ZH ? 0.5 : (l == own ? 1.0 : 0.0);
  }
  return HG_OK;
}

hg_status hg_zones_boundary_samples(hg_zones *z, int64_t *count) {
  if (!z || !count) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = z->n_boundary_samples;
  return HG_OK;
}

double hg_zones_disk_box_area(double x0, double x1, double y0, double y1, double cx, double cy,
                              double r) {
  return disk_box_area(x0, x1, y0, y1, cx, cy, r);
}

} // extern "C"
