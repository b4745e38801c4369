// Zone-label state shared by the zone code (zones.cu) and the resampling
// code (resampling.cu); host only.
#pragma once

#include <cmath>
#include <vector>

#include "hg_gpu.h"

struct hg_zones {
  hg_zones_desc d{};
  // level-set grid
  unsigned N[2] = {0, 0};
  double ls_min[2] = {0, 0}, ls_max[2] = {0, 0}, ls_h = 0.0;
  std::vector<double> phi;      // packing fraction per level-set cell
  std::vector<double> dist;     // signed distance per level-set grid point
  std::vector<int32_t> ls_label;
  std::vector<int32_t> label, prev; // per MPM cell
  struct Box {
    double b[4];
    int32_t c[2];
  };
  std::vector<Box> rzones, direct, ls_rzones;
  int64_t n_boundary_samples = 0;
};

namespace hg {

// MPM cell label at a position (ZoneTools::is...Zone_MPMIndicator,
// ZoneTools.cpp:69-121); -1 outside the MPM grid.
inline int32_t zone_label_at(const hg_zones &z, double x, double y) {
  const int i = (int)std::floor((x - z.d.mpm_grid_min[0]) / z.d.mpm_cell_width);
  const int j = (int)std::floor((y - z.d.mpm_grid_min[1]) / z.d.mpm_cell_width);
  if (i < 0 || j < 0 || i >= z.d.mpm_cells[0] || j >= z.d.mpm_cells[1]) return -1;
  return z.label[(size_t)j * z.d.mpm_cells[0] + i];
}

// identifyInnerContinuumRegion[ExcludingDirectTransitionZones]
// (ZoneTools.cpp:741-798): continuum MPM cells, optionally without those
// that were discrete before the last update.
inline void zone_inner_continuum(const hg_zones &z, bool excluding_direct,
                                 std::vector<hg_zones::Box> &out) {
  out.clear();
  const int mx = z.d.mpm_cells[0], my = z.d.mpm_cells[1];
  const double cw = z.d.mpm_cell_width;
  for (int j = 0; j < my; ++j)
    for (int i = 0; i < mx; ++i) {
      const size_t f = (size_t)j * mx + i;
      if (z.label[f] != HG_ZONE_CONTINUUM) continue;
      if (excluding_direct && z.prev[f] == HG_ZONE_DISCRETE) continue;
      out.push_back({{z.d.mpm_grid_min[0] + i * cw, z.d.mpm_grid_min[1] + j * cw,
                      z.d.mpm_grid_min[0] + (i + 1) * cw, z.d.mpm_grid_min[1] + (j + 1) * cw},
                     {i, j}});
    }
}

} // namespace hg
