// Oracle (test infrastructure only): FP64 restatement of the zone labelling
// of the hybrid method, in the structure of the reference:
//   ZoneTools::init                       ZoneTools.cpp:6-64
//   demWeight / mpmWeight                 ZoneTools.cpp:123-147
//   computePackingFractionForBox          ZoneTools.cpp:149-184
//   updatePackingFraction                 ZoneTools.cpp:186-276
//   addSamplesAlongEdge, updateDistanceField ZoneTools.cpp:278-445
//   estimateLevelSetLevelZoneIndicators   ZoneTools.cpp:447-497
//   sampleMPMLevelZoneIndicators          ZoneTools.cpp:529-665
//   determineMPM/DEM...ToDelete           ZoneTools.cpp:681-739
//   identifyInnerContinuumRegion[...]     ZoneTools.cpp:741-798
//   CUniformGridH2D                       uniformgrid.cpp:41-121
//   redistanceGrid                        levelsetutil.cpp:27-144
//   circleRectangleIntersectionArea       CircleRectangleIntersection.cpp:19-82
// Per-cell id lists with a mailbox, a std::queue sweep and the recursive
// area, as the reference has them; used to check the library's zone code.
#include <algorithm>
#include <cmath>
#include <queue>
#include <vector>

namespace {

enum { ZC = 0, ZD = 1, ZH = 2 };

// circleRectangleIntersectionArea and its helpers
double sec(double h, double r) { return (h < r) ? std::sqrt(r * r - h * h) : 0.0; }
double gint(double x, double h, double r) {
  return .5 * (std::sqrt(1 - x * x / (r * r)) * x * r + r * r * std::asin(x / r) - 2 * h * x);
}
double area_strip(double x0, double x1, double h, double r) {
  if (x0 > x1) std::swap(x0, x1);
  double s = sec(h, r);
  return gint(std::max<double>(-s, std::min<double>(s, x1)), h, r) -
         gint(std::max<double>(-s, std::min<double>(s, x0)), h, r);
}
double area_box(double x0, double x1, double y0, double y1, double r) {
  if (y0 > y1) std::swap(y0, y1);
  if (y0 < 0) {
    if (y1 < 0) return area_box(x0, x1, -y0, -y1, r);
    return area_box(x0, x1, 0, -y0, r) + area_box(x0, x1, 0, y1, r);
  }
  return area_strip(x0, x1, y0, r) - area_strip(x0, x1, y1, r);
}
double disk_box(double x0, double x1, double y0, double y1, double cx, double cy, double r) {
  x0 -= cx;
  x1 -= cx;
  y0 -= cy;
  y1 -= cy;
  return area_box(x0, x1, y0, y1, r);
}

struct UGrid { // CUniformGridH2D
  unsigned res[2];
  double mn[2], cw;
  std::vector<std::vector<int>> ids;
  UGrid(const double m[2], const unsigned r[2], double w) : cw(w) {
    res[0] = r[0];
    res[1] = r[1];
    mn[0] = m[0];
    mn[1] = m[1];
    ids.resize((size_t)r[0] * r[1]);
  }
  void gid(double x, double y, unsigned &i, unsigned &j) const {
    const double a = (x - mn[0]) / cw, b = (y - mn[1]) / cw;
    i = std::max<int>(0, std::min<int>(res[0] - 1, int(std::floor(a))));
    j = std::max<int>(0, std::min<int>(res[1] - 1, int(std::floor(b))));
  }
  void add(double x0, double y0, double x1, double y1, int id) {
    unsigned i0, j0, i1, j1;
    gid(x0, y0, i0, j0);
    gid(x1, y1, i1, j1);
    for (unsigned j = j0; j <= j1; j++)
      for (unsigned i = i0; i <= i1; i++) ids[j * res[0] + i].push_back(id);
  }
};

struct Zones {
  // MPM grid
  double mmin[2], mcw;
  unsigned mcells[2];
  bool direct;
  // DistGrid
  unsigned N[2];
  double dmin[2], dmax[2], dh;
  std::vector<double> minDist, pf;
  std::vector<int> ls, mpm, prev;
  std::vector<std::vector<double>> rz, dz;      // boxes
  std::vector<std::vector<int>> rzi, dzi;       // indices
  int nsamples = 0;
};

double box_fraction(const UGrid &g, double x0, double y0, double x1, double y1,
                    const std::vector<double> &px, const std::vector<double> &py,
                    const std::vector<double> &r, std::vector<int> &mail, int test) {
  double tot = 0.0;
  const double dx = x1 - x0, dy = y1 - y0;
  const double vol = dx * dy;
  unsigned i0, j0, i1, j1;
  g.gid(x0, y0, i0, j0);
  g.gid(x1, y1, i1, j1);
  for (unsigned j = j0; j <= j1; j++)
    for (unsigned i = i0; i <= i1; i++) {
      const std::vector<int> &c = g.ids[j * g.res[0] + i];
      for (size_t q = 0; q < c.size(); q++) {
        if (mail[c[q]] == test) continue;
        mail[c[q]] = test;
        tot += disk_box(x0, x1, y0, y1, px[c[q]], py[c[q]], r[c[q]]);
      }
    }
  return tot / vol;
}

int mpm_label(const Zones &z, double x, double y) {
  const int i = int(std::floor((x - z.mmin[0]) / z.mcw));
  const int j = int(std::floor((y - z.mmin[1]) / z.mcw));
  if (i < int(z.mcells[0]) && j < int(z.mcells[1]) && i >= 0 && j >= 0)
    return z.mpm[j * z.mcells[0] + i];
  return -1;
}

} // namespace

extern "C" {

void *hgo_zones_create(const double mpm_min[2], double mpm_cw, const int cells[2], double ls_cw,
                       int allow_direct) {
  Zones *z = new Zones();
  z->mmin[0] = mpm_min[0];
  z->mmin[1] = mpm_min[1];
  z->mcw = mpm_cw;
  z->mcells[0] = cells[0];
  z->mcells[1] = cells[1];
  z->direct = allow_direct != 0;
  for (int a = 0; a < 2; a++) {
    z->N[a] = unsigned(std::ceil(double(cells[a]) * mpm_cw / ls_cw));
    z->dmin[a] = mpm_min[a];
    z->dmax[a] = z->dmin[a] + ls_cw * double(z->N[a]);
  }
  z->dh = ls_cw;
  z->minDist.assign((z->N[0] + 1) * (z->N[1] + 1), 0.0);
  z->pf.assign(z->N[0] * z->N[1], 0.0);
  z->ls.assign(z->N[0] * z->N[1], ZD);
  z->mpm.assign(cells[0] * cells[1], ZD);
  z->prev.assign(cells[0] * cells[1], ZD);
  return z;
}

void hgo_zones_destroy(void *h) { delete static_cast<Zones *>(h); }

void hgo_zones_packing(void *h, int nd, const double *q3, const double *rad,
                       const unsigned char *fixed, int np, const double *pq, double window,
                       int samples) {
  Zones &z = *static_cast<Zones *>(h);
  std::vector<double> px, py, r;
  for (int b = 0; b < nd; b++) {
    if (fixed && fixed[b]) continue;
    px.push_back(q3[3 * b]);
    py.push_back(q3[3 * b + 1]);
    r.push_back(rad[b]);
  }
  std::fill(z.pf.begin(), z.pf.end(), 0.0);
  std::vector<int> mail(px.size(), 0);
  UGrid g(z.dmin, z.N, z.dh);
  for (size_t i = 0; i < px.size(); i++)
    g.add(px[i] - r[i], py[i] - r[i], px[i] + r[i], py[i] + r[i], int(i));
  int test = 1;
  for (int j = 0; j < int(z.N[1]); j++)
    for (int i = 0; i < int(z.N[0]); i++) {
      double f = 0.0;
      for (int v = 0; v < samples; v++)
        for (int u = 0; u < samples; u++) {
          const double cx = z.dmin[0] + (i + (u + 0.5) / samples) * z.dh;
          const double cy = z.dmin[1] + (j + (v + 0.5) / samples) * z.dh;
          f += box_fraction(g, cx - window * 0.5, cy - window * 0.5, cx + window * 0.5,
                            cy + window * 0.5, px, py, r, mail, test++);
        }
      z.pf[j * z.N[0] + i] = f / (samples * samples);
    }
  for (int p = 0; p < np; p++) {
    const double x = pq[2 * p] - z.dmin[0], y = pq[2 * p + 1] - z.dmin[1];
    const double xl = x - window * 0.5, yl = y - window * 0.5;
    const double xh = x + window * 0.5, yh = y + window * 0.5;
    const int gi0 = int(std::floor(xl / z.dh)), gj0 = int(std::floor(yl / z.dh));
    const int gi1 = int(std::floor(xh / z.dh)), gj1 = int(std::floor(yh / z.dh));
    for (int j = gj0; j <= gj1; j++)
      for (int i = gi0; i <= gi1; i++)
        if (i > 0 && j > 0 && i < int(z.N[0]) && j < int(z.N[1])) z.pf[j * z.N[0] + i] = 1.0;
  }
}

void hgo_zones_distance(void *h, double thr) {
  Zones &z = *static_cast<Zones *>(h);
  const unsigned Nx = z.N[0], Ny = z.N[1];
  std::vector<double> sx, sy;
  auto samples = [&](double ax, double ay, double bx, double by) {
    for (int i = 0; i < 4; i++) {
      const double s = (i + 0.5) / 4;
      sx.push_back((1.0 - s) * ax + s * bx);
      sy.push_back((1.0 - s) * ay + s * by);
    }
  };
  for (int j = 0; j <= int(Ny); j++)
    for (int i = 0; i < int(Nx); i++) {
      const double cl = z.dmin[0] + i * z.dh, cr = z.dmin[0] + (i + 1) * z.dh;
      const double ct = z.dmin[1] + (j + 1) * z.dh;
      const int c = j * Nx + i, top = (j - 1) * int(Nx) + i;
      bool add;
      if (j == 0) add = z.pf[c] > thr;
      else if (j == int(Ny)) add = z.pf[top] > thr;
      else add = (z.pf[top] > thr && z.pf[c] <= thr) || (z.pf[top] <= thr && z.pf[c] > thr);
      if (add) samples(cl, ct, cr, ct);
    }
  for (int j = 0; j < int(Ny); j++)
    for (int i = 0; i <= int(Nx); i++) {
      const double cl = z.dmin[0] + i * z.dh;
      const double cb = z.dmin[1] + j * z.dh, ct = z.dmin[1] + (j + 1) * z.dh;
      const int c = j * Nx + i, left = j * int(Nx) + (i - 1);
      bool add;
      if (i == 0) add = z.pf[c] > thr;
      else if (i == int(Nx)) add = z.pf[left] > thr;
      else add = (z.pf[left] > thr && z.pf[c] <= thr) || (z.pf[left] <= thr && z.pf[c] > thr);
      if (add) samples(cl, cb, cl, ct);
    }
  z.nsamples = int(sx.size());
  // redistanceGrid
  const int npts = (Nx + 1) * (Ny + 1);
  std::vector<double> ad(npts, 1.0e10);
  std::vector<int> cp(npts, -1);
  for (unsigned p = 0; p < sx.size(); p++) {
    const double r = 3.0 * z.dh;
    const double x0 = sx[p] - r, y0 = sy[p] - r, x1 = sx[p] + r, y1 = sy[p] + r;
    const int i0 = std::max<int>(0, std::min<int>(Nx, int(std::floor((Nx) * (x0 - z.dmin[0]) / (z.dmax[0] - z.dmin[0])))));
    const int j0 = std::max<int>(0, std::min<int>(Ny, int(std::floor((Ny) * (y0 - z.dmin[1]) / (z.dmax[1] - z.dmin[1])))));
    const int i1 = std::max<int>(0, std::min<int>(Nx, int(std::ceil((Nx) * (x1 - z.dmin[0]) / (z.dmax[0] - z.dmin[0])))));
    const int j1 = std::max<int>(0, std::min<int>(Ny, int(std::ceil((Ny) * (y1 - z.dmin[1]) / (z.dmax[1] - z.dmin[1])))));
    for (int j = j0; j <= j1; j++)
      for (int i = i0; i <= i1; i++) {
        const unsigned f = j * (Nx + 1) + i;
        const double gx = (z.dmax[0] - z.dmin[0]) * double(i) / double(Nx) + z.dmin[0];
        const double gy = (z.dmax[1] - z.dmin[1]) * double(j) / double(Ny) + z.dmin[1];
        const double ex = gx - sx[p], ey = gy - sy[p];
        const double d = std::sqrt(ex * ex + ey * ey);
        if (d < ad[f]) {
          ad[f] = d;
          cp[f] = int(p);
        }
      }
  }
  std::queue<unsigned> q;
  for (int i = 0; i < npts; i++)
    if (cp[i] >= 0) q.push(i);
  while (!q.empty()) {
    const unsigned id = q.front();
    q.pop();
    const int c = cp[id];
    const unsigned gi = id % (Nx + 1), gj = id / (Nx + 1);
    int nb[4];
    nb[0] = (gi > 0) ? int(gj * (Nx + 1) + gi - 1) : -1;
    nb[1] = (gj > 0) ? int((gj - 1) * (Nx + 1) + gi) : -1;
    nb[2] = (int(gi) < int(Nx)) ? int(gj * (Nx + 1) + gi + 1) : -1;
    nb[3] = (int(gj) < int(Ny)) ? int((gj + 1) * (Nx + 1) + gi) : -1;
    for (int l = 0; l < 4; l++) {
      if (nb[l] < 0) continue;
      const int i = nb[l] % (Nx + 1), j = nb[l] / (Nx + 1);
      const double gx = (z.dmax[0] - z.dmin[0]) * double(i) / double(Nx) + z.dmin[0];
      const double gy = (z.dmax[1] - z.dmin[1]) * double(j) / double(Ny) + z.dmin[1];
      const double ex = gx - sx[c], ey = gy - sy[c];
      const double d = std::sqrt(ex * ex + ey * ey);
      if (d < ad[nb[l]] || cp[nb[l]] < 0) {
        ad[nb[l]] = d;
        cp[nb[l]] = c;
        q.push(nb[l]);
      }
    }
  }
  for (int i = 0; i < npts; i++) z.minDist[i] = ad[i];
  std::vector<int> flag(npts, 0);
  for (int j = 0; j < int(Ny); j++)
    for (int i = 0; i < int(Nx); i++) {
      const int bl = j * (Nx + 1) + i, br = bl + 1, tl = (j + 1) * (Nx + 1) + i, tr = tl + 1;
      if (z.pf[j * Nx + i] > thr) {
        for (int k : {bl, br, tl, tr}) {
          z.minDist[k] = std::fabs(z.minDist[k]);
          flag[k] = 1;
        }
      }
    }
  for (int i = 0; i < npts; i++)
    if (flag[i] == 0) z.minDist[i] = -std::fabs(z.minDist[i]);
}

void hgo_zones_labels(void *h, double level, double half) {
  Zones &z = *static_cast<Zones *>(h);
  const unsigned Nx = z.N[0], Ny = z.N[1];
  for (int j = 0; j < int(Ny); j++)
    for (int i = 0; i < int(Nx); i++) {
      const int fl = j * (Nx + 1) + i, fr = fl + 1, bl = (j + 1) * (Nx + 1) + i, br = bl + 1;
      const double mn = std::min<double>(std::min<double>(z.minDist[fl], z.minDist[fr]),
                                         std::min<double>(z.minDist[bl], z.minDist[br]));
      const double mx = std::max<double>(std::max<double>(z.minDist[fl], z.minDist[fr]),
                                         std::max<double>(z.minDist[bl], z.minDist[br]));
      int &l = z.ls[j * Nx + i];
      if (mx <= level - half) l = ZD;
      else if (mn >= level + half) l = ZC;
      else l = ZH;
    }
  z.prev = z.mpm;
  z.rz.clear();
  z.rzi.clear();
  z.dz.clear();
  z.dzi.clear();
  for (int j = 0; j < int(z.mcells[1]); j++)
    for (int i = 0; i < int(z.mcells[0]); i++) {
      const double ci = double(i), cj = double(j);
      const double x0 = z.mmin[0] + ci * z.mcw, y0 = z.mmin[1] + cj * z.mcw;
      const double x1 = z.mmin[0] + (ci + 1.0) * z.mcw, y1 = z.mmin[1] + (cj + 1.0) * z.mcw;
      int u0 = int(std::floor((x0 - z.dmin[0]) / z.dh)), v0 = int(std::floor((y0 - z.dmin[1]) / z.dh));
      int u1 = int(std::floor((x1 - z.dmin[0]) / z.dh)), v1 = int(std::floor((y1 - z.dmin[1]) / z.dh));
      u0 = std::min<int>(Nx - 1, std::max<int>(0, u0));
      v0 = std::min<int>(Ny - 1, std::max<int>(0, v0));
      u1 = std::min<int>(Nx - 1, std::max<int>(0, u1));
      v1 = std::min<int>(Ny - 1, std::max<int>(0, v1));
      int nh = 0, nc = 0, nd = 0;
      for (int v = v0; v <= v1; v++)
        for (int u = u0; u <= u1; u++) {
          const int l = z.ls[v * Nx + u];
          if (l == ZC) nc++;
          else if (l == ZD) nd++;
          else if (l == ZH) nh++;
        }
      const int f = j * z.mcells[0] + i;
      const std::vector<double> box{x0, y0, x1, y1};
      const std::vector<int> idx{i, j};
      auto hybrid = [&]() {
        z.mpm[f] = ZH;
        z.rz.push_back(box);
        z.rzi.push_back(idx);
      };
      if (nh > 0) {
        hybrid();
      } else if (nd > 0 && nc > 0) {
        hybrid();
      } else if (nd > 0) {
        if (z.direct || z.prev[f] == ZD || z.prev[f] == ZH) z.mpm[f] = ZD;
        else hybrid();
      } else if (nc > 0) {
        if (z.direct) {
          z.mpm[f] = ZC;
          if (z.prev[f] == ZD) {
            z.dz.push_back(box);
            z.dzi.push_back(idx);
          }
        } else if (z.prev[f] == ZC || z.prev[f] == ZH) {
          z.mpm[f] = ZC;
        } else {
          hybrid();
        }
      }
    }
}

void hgo_zones_get(void *h, double *pf, double *dist, int *ls, int *mpm) {
  Zones &z = *static_cast<Zones *>(h);
  if (pf) std::copy(z.pf.begin(), z.pf.end(), pf);
  if (dist) std::copy(z.minDist.begin(), z.minDist.end(), dist);
  if (ls) std::copy(z.ls.begin(), z.ls.end(), ls);
  if (mpm) std::copy(z.mpm.begin(), z.mpm.end(), mpm);
}

int hgo_zones_nsamples(void *h) { return static_cast<Zones *>(h)->nsamples; }

// which: 0 reconciliation, 1 direct transition, 2 inner continuum,
// 3 inner continuum excluding direct transitions
int hgo_zones_list(void *h, int which, double *boxes, int *cells) {
  Zones &z = *static_cast<Zones *>(h);
  std::vector<std::vector<double>> b;
  std::vector<std::vector<int>> c;
  if (which == 0) {
    b = z.rz;
    c = z.rzi;
  } else if (which == 1) {
    b = z.dz;
    c = z.dzi;
  } else {
    for (int j = 0; j < int(z.mcells[1]); j++)
      for (int i = 0; i < int(z.mcells[0]); i++) {
        const int f = j * z.mcells[0] + i;
        if (z.mpm[f] != ZC) continue;
        if (which == 3 && z.prev[f] == ZD) continue;
        b.push_back({z.mmin[0] + i * z.mcw, z.mmin[1] + j * z.mcw, z.mmin[0] + (i + 1) * z.mcw,
                     z.mmin[1] + (j + 1) * z.mcw});
        c.push_back({i, j});
      }
  }
  for (size_t k = 0; k < b.size(); k++) {
    if (boxes)
      for (int e = 0; e < 4; e++) boxes[4 * k + e] = b[k][e];
    if (cells) {
      cells[2 * k] = c[k][0];
      cells[2 * k + 1] = c[k][1];
    }
  }
  return int(b.size());
}

int hgo_zones_to_delete(void *h, int kind, int n, const double *x, int stride,
                        const unsigned char *fixed, int *ids) {
  Zones &z = *static_cast<Zones *>(h);
  int c = 0;
  for (int p = 0; p < n; p++) {
    if (kind == 1 && fixed && fixed[p]) continue;
    const int l = mpm_label(z, x[stride * p], x[stride * p + 1]);
    if (l < 0 || l == (kind == 0 ? ZD : ZC)) ids[c++] = p;
  }
  return c;
}

void hgo_zones_weights(void *h, int kind, int n, const double *x, int stride, double *w) {
  Zones &z = *static_cast<Zones *>(h);
  for (int p = 0; p < n; p++) {
    const int l = mpm_label(z, x[stride * p], x[stride * p + 1]);
    if (l == ZH) w[p] = 0.5;
    else if (l == (kind == 0 ? ZC : ZD)) w[p] = 1.0;
    else w[p] = 0.0;
  }
}

void hgo_zones_set_labels(void *h, const int *mpm) {
  Zones &z = *static_cast<Zones *>(h);
  std::copy(mpm, mpm + z.mpm.size(), z.mpm.begin());
}

double hgo_disk_box_area(double x0, double x1, double y0, double y1, double cx, double cy,
                         double r) {
  return disk_box(x0, x1, y0, y1, cx, cy, r);
}

} // extern "C"
