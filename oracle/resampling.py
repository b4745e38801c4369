"""Oracle (test infrastructure only): pure-Python restatement of the hybrid
method's resampling step, for small scenes.

Follows, in the reference's order and FP64 evaluation order:
  HybridGrains2DSim::updateHybridStates_poorman  HybridGrains2DSim.cpp:327-536
  ResamplingTools (insertion, quantities, deletion) ResamplingTools.cpp:16-725
  CAvoidAVoid::avoidAVoid / randomFillRegion / conflictCheck
                                                 AvoidAvoid.cpp:103-183, 261-298
  Grid (mass-weighted fields, interpolation)     Grid.cpp:45-348
  ConstitutiveModel::computeStrainFromCauchyStress ConstitutiveModel.cpp:99-117
  randomMT (MT19937, seed 4357)                  random.c:58-126
and libstdc++'s std::default_random_engine (minstd_rand0, seed 1) with
std::normal_distribution (Marsaglia polar method over generate_canonical),
which ResamplingTools uses for grain radii (ResamplingTools.h:107-108).
The zone labels come from the C++ oracle (oracle.Zones).
"""
import math
import struct

import numpy as np

CONTINUUM, DISCRETE, HYBRID = 0, 1, 2


def f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


class MT:
    """randomMT / randomMT_i of random.c."""

    def __init__(self):
        self.mt = [0] * 624
        self.mti = 625

    def seed(self, s):
        self.mt[0] = s & 0xFFFFFFFF
        for i in range(1, 624):
            self.mt[i] = (69069 * self.mt[i - 1]) & 0xFFFFFFFF
        self.mti = 624

    def u32(self):
        mt = self.mt
        if self.mti >= 624:
            if self.mti == 625:
                self.seed(4357)
            for kk in range(624 - 397):
                y = (mt[kk] & 0x80000000) | (mt[kk + 1] & 0x7FFFFFFF)
                mt[kk] = mt[kk + 397] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            for kk in range(624 - 397, 623):
                y = (mt[kk] & 0x80000000) | (mt[kk + 1] & 0x7FFFFFFF)
                mt[kk] = mt[kk + (397 - 624)] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            y = (mt[623] & 0x80000000) | (mt[0] & 0x7FFFFFFF)
            mt[623] = mt[396] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.mti = 0
        y = mt[self.mti]
        self.mti += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def f32(self):
        # (float)y * (float)2.3283064365386963e-10, in single precision
        return f32(f32(float(self.u32())) * f32(2.3283064365386963e-10))


class Normal:
    """std::normal_distribution<double>(mean, std) driven by minstd_rand0."""

    R = 2147483646.0  # max - min + 1 of minstd_rand0

    def __init__(self, mean, std):
        self.x = 1  # minstd_rand0 default seed (shared engine, see reset)
        self.mean, self.std = mean, std
        self.saved = None

    def reset_params(self, mean, std):
        self.mean, self.std = mean, std
        self.saved = None

    def _engine(self):
        self.x = (16807 * self.x) % 2147483647
        return self.x

    def _canonical(self):
        # generate_canonical<double, 53>: two engine calls of 30 usable bits
        s = float(self._engine() - 1) * 1.0
        s += float(self._engine() - 1) * self.R
        r = s / (self.R * self.R)
        if r >= 1.0:
            r = math.nextafter(1.0, 0.0)
        return r

    def __call__(self):
        if self.saved is not None:
            ret, self.saved = self.saved, None
        else:
            while True:
                x = 2.0 * self._canonical() - 1.0
                y = 2.0 * self._canonical() - 1.0
                r2 = x * x + y * y
                if not (r2 > 1.0 or r2 == 0.0):
                    break
            mult = math.sqrt(-2 * math.log(r2) / r2)
            self.saved = x * mult
            ret = y * mult
        return ret * self.std + self.mean


class UGrid:
    """CUniformGridH2D."""

    def __init__(self, mn, res, cw):
        self.mn, self.res, self.cw = mn, (max(res[0], 1), max(res[1], 1)), cw
        self.cells = [[] for _ in range(self.res[0] * self.res[1])]

    def gid(self, x, y):
        i = max(0, min(self.res[0] - 1, int(math.floor((x - self.mn[0]) / self.cw))))
        j = max(0, min(self.res[1] - 1, int(math.floor((y - self.mn[1]) / self.cw))))
        return i, j

    def add_box(self, x0, y0, x1, y1, idx):
        i0, j0 = self.gid(x0, y0)
        i1, j1 = self.gid(x1, y1)
        for j in range(j0, j1 + 1):
            for i in range(i0, i1 + 1):
                self.cells[j * self.res[0] + i].append(idx)

    def add_point(self, x, y, idx):
        i, j = self.gid(x, y)
        self.cells[j * self.res[0] + i].append(idx)

    def ids(self, i, j):
        if i >= self.res[0] or j >= self.res[1]:
            return []
        return self.cells[j * self.res[0] + i]

    def each(self, x0, y0, x1, y1):
        i0, j0 = self.gid(x0, y0)
        i1, j1 = self.gid(x1, y1)
        for j in range(j0, j1 + 1):
            for i in range(i0, i1 + 1):
                yield from self.ids(i, j)


def lin_n(x):
    a = abs(x)
    return 1.0 - a if a < 1.0 else 0.0


def lin_integral(xp, hl, xi, w):
    diff = abs(xp - xi)
    if diff >= w + hl:
        return 0.0
    if diff >= w - hl:
        return (w + hl - diff) * (w + hl - diff) / (2.0 * w)
    if diff >= hl:
        return 2.0 * hl * (1.0 - diff / w)
    return 2.0 * hl - (hl * hl + diff * diff) / w


def stencil(basis, x, y, hl, gx, gy, h):
    if basis == 0:
        x0, y0 = int(math.floor((x - gx) / h)), int(math.floor((y - gy) / h))
        return x0, y0, x0 + 1, y0 + 1
    return (int(math.floor(((x - hl) - gx) / h)), int(math.floor(((y - hl) - gy) / h)),
            int(math.ceil(((x + hl) - gx) / h)), int(math.ceil(((y + hl) - gy) / h)))


def weight(basis, x, y, hl, ix, iy, gx, gy, h):
    if basis == 0:
        return lin_n(((x - h * ix) - gx) / h) * lin_n(((y - h * iy) - gy) / h)
    xi, yi = h * ix + gx, h * iy + gy
    Vp = 4.0 * hl * hl
    return lin_integral(x, hl, xi, h) * lin_integral(y, hl, yi, h) / Vp


def det2(a):
    return a[0] * a[3] - a[1] * a[2]


class Resampler:
    """ResamplingTools + the resampling part of updateHybridStates_poorman."""

    def __init__(self, gmin, gmax, cw, cells, basis, size, density, r_mean, r_std, rho_dem,
                 kappa, mu, stress_free=False, hom_stress=False, hom_vel=False):
        self.gmin, self.gmax, self.cw, self.cells = gmin, gmax, cw, cells
        self.basis, self.size, self.density = basis, size, density
        self.r_mean, self.r_std, self.rho_dem = r_mean, r_std, rho_dem
        self.kappa, self.mu = kappa, mu
        self.stress_free, self.hom_stress, self.hom_vel = stress_free, hom_stress, hom_vel
        self.mt = MT()
        self.normal = Normal(r_mean, r_std)
        self.grid_h = (gmax[0] - gmin[0]) / cells[0]
        nn = (cells[0] + 1) * (cells[1] + 1)
        self.hs = [0.0] * (4 * nn)
        self.hv = [0.0] * (2 * nn)

    # ---- state -------------------------------------------------------------
    def set_points(self, q0, q, v, m, vol, m0, vol0, hl, be, J, jh=None):
        n = len(m)
        self.P = {"q0": [list(map(float, r)) for r in q0], "q": [list(map(float, r)) for r in q],
                  "v": [list(map(float, r)) for r in v], "m": list(map(float, m)),
                  "vol": list(map(float, vol)), "m0": list(map(float, m0)),
                  "vol0": list(map(float, vol0)), "w": [1.0] * n, "hl": list(map(float, hl)),
                  "be": [list(map(float, r)) for r in be], "J": list(map(float, J)),
                  "jh": [0] * n if jh is None else list(map(int, jh))}

    def set_grains(self, q0, q, v, r, M0, fixed):
        self.G = {"q0": [list(map(float, x)) for x in q0], "q": [list(map(float, x)) for x in q],
                  "v": [list(map(float, x)) for x in v], "r": list(map(float, r)),
                  "M0": [list(map(float, x)) for x in M0], "w": [1.0] * len(r),
                  "fixed": [int(f) for f in fixed]}

    def set_homogenized(self, stress, vel):
        self.hs = list(map(float, np.ravel(stress)))
        self.hv = list(map(float, np.ravel(vel)))

    # ---- avoid-a-void ----------------------------------------------------------
    def _fill(self, regions, mean_r, px, py, rad, sampler):
        if len(regions) == 0:
            return
        lo = [regions[0][0], regions[0][1]]
        up = [regions[0][2], regions[0][3]]
        for b in regions[1:]:
            lo = [min(lo[0], b[0]), min(lo[1], b[1])]
            up = [max(up[0], b[2]), max(up[1], b[3])]
        g0 = (lo[0] - 6.0 * mean_r, lo[1] - 6.0 * mean_r)
        g1 = (up[0] + 6.0 * mean_r, up[1] + 6.0 * mean_r)
        cw = 4.0 * mean_r
        grid = UGrid(g0, (int(math.ceil((g1[0] - g0[0]) / cw)), int(math.ceil((g1[1] - g0[1]) / cw))),
                     cw)
        for b in range(len(px)):
            grid.add_box(px[b] - rad[b], py[b] - rad[b], px[b] + rad[b], py[b] + rad[b], b)
        for reg in regions:
            dx, dy = reg[2] - reg[0], reg[3] - reg[1]
            for _ in range(16):
                x = self.mt.f32() * dx + reg[0]
                y = self.mt.f32() * dy + reg[1]
                r = sampler()
                hit = False
                seen = set()
                for idx in grid.each(x - r, y - r, x + r, y + r):
                    if idx in seen:
                        continue
                    seen.add(idx)
                    ex, ey = px[idx] - x, py[idx] - y
                    if math.sqrt(ex * ex + ey * ey) < (rad[idx] + r) * 0.97:
                        hit = True
                        break
                if hit:
                    continue
                px.append(x)
                py.append(y)
                rad.append(r)
                grid.add_box(x - r, y - r, x + r, y + r, len(px) - 1)

    def _insert_points(self, zones):
        P = self.P
        rp = 0.5 * self.size
        n = len(P["m"])
        px = [q[0] for q in P["q"]]
        py = [q[1] for q in P["q"]]
        rad = [rp] * n
        self._fill(zones, rp, px, py, rad, lambda: rp)
        for k in range(n, len(px)):
            x = [px[k], py[k]]
            P["q0"].append(list(x))
            P["q"].append(list(x))
            P["v"].append([0.0, 0.0])
            for f in ("m", "vol", "m0", "vol0"):
                P[f].append(0.0)
            P["w"].append(1.0)
            P["hl"].append(self.size * 0.5)
            P["be"].append([1.0, 0.0, 0.0, 1.0])
            P["J"].append(1.0)
            P["jh"].append(0)
        self.stats["points_inserted"] += len(px) - n
        return n

    def _insert_grains(self, zones):
        G = self.G
        n = len(G["r"])
        px = [q[0] for q in G["q"]]
        py = [q[1] for q in G["q"]]
        rad = list(G["r"])
        lo, hi = self.r_mean - 2.0 * self.r_std, self.r_mean + 2.0 * self.r_std
        r_mean = self.r_mean
        unset = self.r_mean < 0.0
        if unset:
            r_mean = rad[0]
            self.normal.reset_params(rad[0], 0.0)

        def sample():
            if unset:
                return self.normal()
            r = -1.0e33
            while r < lo or r > hi:
                r = self.normal()
            return r

        self._fill(zones, r_mean, px, py, rad, sample)
        for k in range(n, len(px)):
            r = rad[k]
            m = self.rho_dem * math.pi * r * r
            inertia = 0.5 * m * r * r
            G["q"].append([px[k], py[k], 0.0])
            G["q0"].append([px[k], py[k], 0.0])
            G["v"].append([0.0, 0.0, 0.0])
            G["r"].append(r)
            G["M0"].append([m, m, inertia])
            G["w"].append(1.0)
            G["fixed"].append(0)
        self.stats["grains_inserted"] += len(px) - n
        return n

    # ---- quantities ----------------------------------------------------------
    def _grids(self):
        cont = UGrid(self.gmin, self.cells, self.cw)
        disc = UGrid(self.gmin, self.cells, self.cw)
        for k, q in enumerate(self.P["q"]):
            cont.add_point(q[0], q[1], k)
        for k, q in enumerate(self.G["q"]):
            disc.add_point(q[0], q[1], k)
        return cont, disc

    def _nodes(self, x0, y0, x1, y1):
        # the reference loops over the stencil with unsigned bounds: a
        # negative start runs no iteration
        if x0 < 0 or y0 < 0:
            return []
        return [(ix, iy) for iy in range(y0, min(y1, self.cells[1]) + 1)
                for ix in range(x0, min(x1, self.cells[0]) + 1)]

    def _interp(self, x, y, hl, h, field, length):
        out = [0.0] * length
        x0, y0, x1, y1 = stencil(self.basis, x, y, hl, self.gmin[0], self.gmin[1], h)
        for ix, iy in self._nodes(x0, y0, x1, y1):
            w = weight(self.basis, x, y, hl, ix, iy, self.gmin[0], self.gmin[1], h)
            node = iy * (self.cells[0] + 1) + ix
            for c in range(length):
                out[c] += w * field[node * length + c]
        return out

    def _strain(self, s):
        T = s[0] + s[3]
        J = 0.5 * (T / self.kappa + math.sqrt((T * T) / (self.kappa * self.kappa) + 4.0))
        dev = [s[0] - T * 1.0 / 2.0, s[1] - T * 0.0 / 2.0, s[2] - T * 0.0 / 2.0,
               s[3] - T * 1.0 / 2.0]
        dev = [J * d / self.mu for d in dev]
        t = math.sqrt(1.0 - det2(dev))
        return J, [dev[0] + t * 1.0, dev[1] + t * 0.0, dev[2] + t * 0.0, dev[3] + t * 1.0]

    def _hybrid_points(self, zone_cells, before, after, g_before, cont, disc):
        P, G = self.P, self.G
        cell_volume = self.cw * self.cw
        mass_per_cell = self.density * cell_volume
        for (i, j) in zone_cells:
            ids = cont.ids(int(i), int(j))
            for k in ids:
                P["m0"][k] = mass_per_cell / len(ids)
                P["vol0"][k] = cell_volume / len(ids)
        sigma, max_dist = 0.5 * self.size, 3.0 * self.size
        hh = self.cw * 0.25
        for p in range(before, after):
            x, y = P["q"][p]
            vs, q0s, Js, bes, ws, nn = [0.0, 0.0], [0.0, 0.0], 0.0, [0.0] * 4, 0.0, 0
            for k in cont.each(x - max_dist, y - max_dist, x + max_dist, y + max_dist):
                if k >= before:
                    continue
                ex, ey = P["q"][k][0] - x, P["q"][k][1] - y
                d = math.sqrt(ex * ex + ey * ey)
                if d <= max_dist:
                    w = math.exp(-(d * d) / (2.0 * sigma * sigma))
                    vs = [vs[0] + P["v"][k][0] * w, vs[1] + P["v"][k][1] * w]
                    q0s = [q0s[0] + P["q0"][k][0] * w, q0s[1] + P["q0"][k][1] * w]
                    Js += P["J"][k] * w
                    bes = [bes[c] + P["be"][k][c] * w for c in range(4)]
                    ws += w
                    nn += 1
            stress = self._interp(x, y, hh, self.cw, self.hs, 4) if self.hom_stress else [0.0] * 4
            hvel = self._interp(x, y, hh, self.cw, self.hv, 2) if self.hom_vel else [0.0, 0.0]
            if nn == 0:
                Jn, ben = 1.0, [1.0, 0.0, 0.0, 1.0]
            else:
                Jn = Js / ws
                ben = [b / ws for b in bes]
                sd = math.sqrt(det2(ben))
                ben = [b / sd for b in ben]
            for k in disc.each(x - max_dist, y - max_dist, x + max_dist, y + max_dist):
                if k >= g_before:
                    continue
                ex, ey = G["q"][k][0] - x, G["q"][k][1] - y
                d = math.sqrt(ex * ex + ey * ey)
                if d <= max_dist:
                    w = math.exp(-(d * d) / (2.0 * sigma * sigma))
                    vs = [vs[0] + G["v"][k][0] * w, vs[1] + G["v"][k][1] * w]
                    q0s = [q0s[0] + G["q0"][k][0] * w, q0s[1] + G["q0"][k][1] * w]
                    ws += w
            if ws == 0.0:
                vn, q0n = [0.0, 0.0], [x, y]
            else:
                vn, q0n = [vs[0] / ws, vs[1] / ws], [q0s[0] / ws, q0s[1] / ws]
            P["q0"][p] = q0n
            P["v"][p] = hvel if self.hom_vel else vn
            if self.hom_stress:
                Jn, ben = self._strain(stress)
                P["J"][p] = Jn
            else:
                P["J"][p] = 1.0 if self.stress_free else Jn
            P["be"][p] = ben

    def _grains(self, before, after, p_before, cont, disc):
        P, G = self.P, self.G
        sigma, max_dist = self.r_mean, 6.0 * self.r_mean
        for b in range(before, after):
            x, y = G["q"][b][0], G["q"][b][1]
            vs, q0s, ws = [0.0] * 3, [0.0] * 3, 0.0
            for k in disc.each(x - max_dist, y - max_dist, x + max_dist, y + max_dist):
                if k >= before:
                    continue
                ex, ey = G["q"][k][0] - x, G["q"][k][1] - y
                d = math.sqrt(ex * ex + ey * ey)
                if d <= max_dist:
                    w = math.exp(-(d * d) / (2.0 * sigma * sigma))
                    vs = [vs[c] + G["v"][k][c] * w for c in range(3)]
                    q0s = [q0s[c] + G["q0"][k][c] * w for c in range(3)]
                    ws += w
            for k in cont.each(x - max_dist, y - max_dist, x + max_dist, y + max_dist):
                if k >= p_before:
                    continue
                ex, ey = P["q"][k][0] - x, P["q"][k][1] - y
                d = math.sqrt(ex * ex + ey * ey)
                if d <= max_dist:
                    w = math.exp(-(d * d) / (2.0 * sigma * sigma))
                    vs = [vs[0] + P["v"][k][0] * w, vs[1] + P["v"][k][1] * w, vs[2] + 0.0 * w]
                    q0s = [q0s[0] + P["q0"][k][0] * w, q0s[1] + P["q0"][k][1] * w,
                           q0s[2] + 0.0 * w]
                    ws += w
            if ws == 0.0:
                G["v"][b] = [0.0, 0.0, 0.0]
                G["q0"][b] = [x, y, 0.0]
            else:
                G["v"][b] = [vs[c] / ws for c in range(3)]
                G["q0"][b] = [q0s[c] / ws for c in range(3)]

    def _field(self, n, vals, length, dflt):
        P = self.P
        nx, ny = self.cells
        nn = (nx + 1) * (ny + 1)
        mass = [0.0] * nn
        out = [0.0] * (nn * length)
        h1 = P["hl"][0] if P["hl"] else 0.0
        for p in range(n):
            x, y = P["q"][p]
            x0, y0, x1, y1 = stencil(self.basis, x, y, h1, self.gmin[0], self.gmin[1], self.grid_h)
            for ix, iy in self._nodes(x0, y0, x1, y1):
                w = weight(self.basis, x, y, h1, ix, iy, self.gmin[0], self.gmin[1], self.grid_h)
                node = iy * (nx + 1) + ix
                mass[node] += w * P["m"][p]
                for c in range(length):
                    out[node * length + c] += w * P["m"][p] * vals[p][c]
        for node in range(nn):
            for c in range(length):
                if mass[node] > 0.0:
                    out[node * length + c] /= mass[node]
                else:
                    out[node * length + c] = dflt[c]
        return out

    def _inner_points(self, before, after, cont):
        P = self.P
        fJ = self._field(before, [[j] for j in P["J"]], 1, [1.0])
        fv = self._field(before, P["v"], 2, [0.0, 0.0])
        fb = self._field(before, P["be"], 4, [1.0, 0.0, 0.0, 1.0])
        sigma, rr = 0.5 * self.size, 2.0 * self.size
        for i in range(before, after):
            x, y = P["q"][i]
            tm = tv = ws = 0.0
            q0s = [0.0, 0.0]
            nb = []
            for k in cont.each(x - rr, y - rr, x + rr, y + rr):
                if k >= i:
                    continue
                ex, ey = x - P["q"][k][0], y - P["q"][k][1]
                d2 = ex * ex + ey * ey
                if d2 < rr * rr:
                    w = math.exp(-(d2 * d2) / (2.0 * sigma * sigma))
                    ws += w
                    q0s = [q0s[0] + w * P["q0"][k][0], q0s[1] + w * P["q0"][k][1]]
                    nb.append(k)
                    tm += P["m0"][k]
                    tv += P["vol0"][k]
            count = len(nb)
            with np.errstate(invalid="ignore", divide="ignore"):
                P["q0"][i] = [float(np.float64(q0s[0]) / np.float64(ws)),
                              float(np.float64(q0s[1]) / np.float64(ws))]
            P["m0"][i] = tm / (count + 1.0)
            P["vol0"][i] = tv / (count + 1.0)
            factor = float(count) / float(count + 1.0)
            for k in nb:
                P["m0"][k] *= factor
                P["vol0"][k] *= factor
        h1 = P["hl"][0] if P["hl"] else 0.0
        for p in range(before, after):
            x, y = P["q"][p]
            J = self._interp(x, y, h1, self.grid_h, fJ, 1)[0]
            be = self._interp(x, y, h1, self.grid_h, fb, 4)
            sd = math.sqrt(det2(be))
            be = [b / sd for b in be]
            vel = self._interp(x, y, h1, self.grid_h, fv, 2)
            P["v"][p] = vel
            if self.stress_free:
                P["J"][p], P["be"][p] = 1.0, [1.0, 0.0, 0.0, 1.0]
            else:
                P["J"][p], P["be"][p] = J, be

    # ---- deletion and weights ---------------------------------------------------
    def _label(self, labels, x, y):
        i = int(math.floor((x - self.gmin[0]) / self.cw))
        j = int(math.floor((y - self.gmin[1]) / self.cw))
        if i < 0 or j < 0 or i >= self.cells[0] or j >= self.cells[1]:
            return -1
        return int(labels[j * self.cells[0] + i])

    def _delete(self, labels):
        P, G = self.P, self.G
        keep = [not (self._label(labels, q[0], q[1]) in (-1, DISCRETE)) for q in P["q"]]
        self.stats["points_deleted"] += keep.count(False)
        for f in P:
            P[f] = [x for x, k in zip(P[f], keep) if k]
        keepb = []
        for b, q in enumerate(G["q"]):
            if G["fixed"][b]:
                keepb.append(True)
                continue
            keepb.append(not (self._label(labels, q[0], q[1]) in (-1, CONTINUUM)))
        self.dem_map, nxt = [], 0
        for k in keepb:
            self.dem_map.append(nxt if k else -1)
            nxt += 1 if k else 0
        self.stats["grains_deleted"] += keepb.count(False)
        for f in G:
            G[f] = [x for x, k in zip(G[f], keepb) if k]

    def _weights(self, labels):
        P, G = self.P, self.G
        for b, q in enumerate(G["q"]):
            lab = self._label(labels, q[0], q[1])
            G["w"][b] = 0.5 if lab == HYBRID else (1.0 if lab == DISCRETE else 0.0)
        for p, q in enumerate(P["q"]):
            lab = self._label(labels, q[0], q[1])
            P["w"][p] = 0.5 if lab == HYBRID else (1.0 if lab == CONTINUUM else 0.0)
            P["m"][p] = P["m0"][p] * P["w"][p]
            P["vol"][p] = P["vol0"][p] * P["w"][p]

    def run(self, zones, allow_direct):
        """zones: an oracle.Zones after update()."""
        self.stats = dict(points_inserted=0, grains_inserted=0, points_deleted=0,
                          grains_deleted=0)
        rz, rzi = zones.zone_list(0)
        dz, dzi = zones.zone_list(1)
        inner, _ = zones.zone_list(3 if allow_direct else 2)
        labels = zones.fields()["mpm"]
        g_before = self._insert_grains([list(b) for b in rz])
        g_after = len(self.G["r"])
        p_before = self._insert_points([list(b) for b in rz])
        p_mid = len(self.P["m"])
        if allow_direct:
            self._insert_points([list(b) for b in dz])
        p_after = len(self.P["m"])
        i_before = i_after = p_after
        if len(inner):
            i_before = self._insert_points([list(b) for b in inner])
            i_after = len(self.P["m"])
        cont, disc = self._grids()
        if allow_direct:
            self._hybrid_points(rzi, p_before, p_mid, g_before, cont, disc)
            self._hybrid_points(dzi, p_mid, p_after, g_before, cont, disc)
        else:
            self._hybrid_points(rzi, p_before, p_after, g_before, cont, disc)
        self._grains(g_before, g_after, p_before, cont, disc)
        self._inner_points(i_before, i_after, cont)
        self._delete(labels)
        self._weights(labels)
