"""Restatement of the reference's grid-point numbering and neighbour tables.

TEST INFRASTRUCTURE (part of the oracle): only tests/ may import this module.
It is the checker of the integer grid tables the product's builder
(csrc/fim_grid.cpp) produces, never a part of the product path.

What it restates, for the standard recursive construction (gtype 0,
SubdivNum = 2 at every level) and the IJ cell order (curve 0):

* FIMsrc/prep/grid/top_gridpoints.F90:8-108  the 12 icosahedron points and
  their neighbour lists; rotate.F90:8-92 the 10 degree turn about the axis
  (icos.F90:68-70);
* FIMsrc/prep/grid/top_triangles.F90:14-84   the 20 top triangles;
* FIMsrc/prep/grid/icos.F90:126-239          comp_grid (per-triangle sequence
  numbers and buffer offsets) and proc_grid (edge removal, rhombus assembly,
  rhombus offsets), and icos.F90:100-119 (pole numbers, +1 on output);
* FIMsrc/prep/grid/bisect_triangle.F90:134-253, 685-843  bisect_triangle_nasr,
  bisect_r_triangle_nasr, compute_index, row, remove_edge1, remove_edge2,
  combine;
* FIMsrc/prep/grid/middle.F90:23-72          the great-circle midpoint in
  degrees (the degree/radian factor there is 4*atan(1.0) in single precision
  divided by 180 in double, and the end points are converted in place);
* FIMsrc/prep/grid/GridGen.F90:98-217, 503-623  the pattern-based neighbour
  lists (grid_point_type, special_points); with curve 0 the permutation of
  perm.F90:41-72 is the identity;
* FIMsrc/prep/grid/getlvl.F90:145-157        proxs, the neighbour's slot of
  the shared edge; dyn_init.F90:545-549 prox(6) = prox(5) at a pentagon.

Pure Python loops over the recursion: fine up to glvl 6 in a few seconds.
"""
import math

import numpy as np

_PI32 = float(np.float32(4.0) * np.arctan(np.float32(1.0)))  # 4.0*ATAN(1.0), default real


def _middle(p1, p2):
    """middle.F90:23-72; p1 and p2 are converted in place, as the reference
    passes them by reference (deg -> rad -> deg), so they are returned too."""
    d2r = _PI32 / 180.0
    a = [p1[0] * d2r, p1[1] * d2r]
    b = [p2[0] * d2r, p2[1] * d2r]
    x1 = (math.cos(a[0]) * math.cos(a[1]), math.cos(a[0]) * math.sin(a[1]), math.sin(a[0]))
    x2 = (math.cos(b[0]) * math.cos(b[1]), math.cos(b[0]) * math.sin(b[1]), math.sin(b[0]))
    x = [0.5 * (x1[k] + x2[k]) for k in range(3)]
    n = math.sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2])
    x = [v / n for v in x]
    lat = math.atan2(x[2], math.sqrt(x[0] * x[0] + x[1] * x[1]))
    lon = math.atan2(x[1], x[0])
    if lon < -_PI32 / 2.0:
        lon = lon + 2 * _PI32
    return [a[0] / d2r, a[1] / d2r], [b[0] / d2r, b[1] / d2r], [lat / d2r, lon / d2r]


def _rotate_z(latlon_deg, theta_deg):
    """rotate.F90:8-92 with lambda = 0 (a turn of theta about the z axis)."""
    d2r = _PI32 / 180.0
    t = theta_deg * d2r
    st, ct = math.sin(t), math.cos(t)
    la, lo = latlon_deg[0] * d2r, latlon_deg[1] * d2r
    x = (math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la))
    y = (ct * x[0] - st * x[1], st * x[0] + ct * x[1], x[2])
    lat = math.atan2(y[2], math.sqrt(y[0] * y[0] + y[1] * y[1]))
    lon = math.atan2(y[1], y[0])
    if lon < -_PI32 / 2.0:
        lon = lon + 2 * _PI32
    return [lat / d2r, lon / d2r]


def _top_grid():
    """top_gridpoints.F90:8-108: latlon and neighbours (degrees) of the 12 points."""
    lat0, lon0 = 26.5650428671016, -72.0
    top = [{"ll": [0.0, 0.0], "nb": [[0.0, 0.0] for _ in range(6)]} for _ in range(13)]  # 1-based
    top[1]["ll"] = [90.0, 0.0]
    for i in range(1, 6):
        top[1]["nb"][i - 1] = [lat0, lon0 + 72.0 * i]
    for i in range(2, 7):
        top[i]["ll"] = list(top[1]["nb"][i - 2])
        top[i]["nb"][0] = list(top[1]["ll"])
        n = 5 if i - 1 == 1 else i - 1
        top[i]["nb"][1] = list(top[1]["nb"][n - 1])
        n = 2 if i + 1 == 7 else i + 1
        top[i]["nb"][2] = list(top[1]["nb"][n - 1])
    top[7]["ll"] = [-90.0, 0.0]
    for i in range(1, 6):
        top[7]["nb"][i - 1] = [-lat0, lon0 + 36.0 + 72.0 * i]
    for i in range(8, 13):
        top[i]["ll"] = list(top[7]["nb"][i - 8])
        top[i]["nb"][0] = list(top[7]["ll"])
        n = 12 if i - 1 == 7 else i - 1
        top[i]["nb"][1] = list(top[7]["nb"][n - 8])
        n = 8 if i == 12 else i
        top[i]["nb"][2] = list(top[7]["nb"][n - 7])
    for i in range(2, 7):
        n = i + 6
        top[i]["nb"][3] = list(top[n]["ll"])
        top[n]["nb"][3] = list(top[i]["ll"])
        n = 12 if i + 5 == 7 else i + 5
        top[i]["nb"][4] = list(top[n]["ll"])
        top[n]["nb"][4] = list(top[i]["ll"])
    for i in range(1, 13):
        top[i]["ll"] = _rotate_z(top[i]["ll"], 10.0)
        top[i]["nb"] = [_rotate_z(p, 10.0) for p in top[i]["nb"]]
    return top


def _top_triangles(top):
    """top_triangles.F90:14-84: vertex latlons of the 20 triangles (1-based)."""
    tri = [None] * 21
    for i in range(1, 6):
        n = 1 if i + 1 == 6 else i + 1
        tri[i] = [list(top[1]["ll"]), list(top[1]["nb"][i - 1]), list(top[1]["nb"][n - 1])]
    for i in range(6, 11):
        n = 6 if i + 1 == 11 else i + 1
        tri[i] = [list(top[7]["ll"]), list(top[7]["nb"][n - 6]), list(top[7]["nb"][i - 6])]
    for i in range(1, 6):
        tri[i + 10] = [list(top[i + 1]["ll"]), list(top[i + 1]["nb"][4]), list(top[i + 1]["nb"][3])]
    for i in range(8, 13):
        tri[i + 8] = [list(top[i]["ll"]), list(top[i]["nb"][4]), list(top[i]["nb"][3])]
    return tri


class _Icos:
    """comp_grid / proc_grid of icos.F90 over the gp buffer (1-based)."""

    def __init__(self, glvl):
        self.ml = glvl
        self.sl = 2 ** glvl
        sl = self.sl
        self.init_c_sn = (sl + 2) * (sl + 1) // 2 - 1
        buf = 20 * (sl + 2) * (sl + 1) // 2
        self.lat = [0.0] * (buf + 1)
        self.lon = [0.0] * (buf + 1)
        self.seq = [0] * (buf + 1)
        self.offset = 0

    def _row(self, x):
        s = self.init_c_sn - x
        n = (math.isqrt(1 + 8 * s) - 1) // 2  # INT((sqrt(REAL(1+8s))-1)/2), exact here
        return self.sl - n

    def _compute_index(self, a, b, c, delta):
        init_stride = (self.sl + 1) - self._row(a)
        nrtm = (self._row(c) - self._row(a)) // 2
        stride1 = (2 * init_stride - (nrtm - 1)) * nrtm // 2
        stride2 = (2 * (init_stride - 1) - (nrtm - 1)) * nrtm // 2
        a_c = a + stride1
        if delta == 1:
            a_b = (a + b) // 2
            b_c = b + stride2
        else:
            b_c = (b + c) // 2
            a_b = a + stride2
        return a_b, a_c, b_c

    def _store(self, *pts):
        for p in pts:
            k = p["sn"] + self.offset
            self.lat[k], self.lon[k] = p["ll"]
            self.seq[k] = p["sn"]

    def _split(self, a, b, c, clevel, delta):
        ab, ac, bc = self._compute_index(a["sn"], b["sn"], c["sn"], delta)
        a["ll"], b["ll"], m_ab = _middle(a["ll"], b["ll"])
        a["ll"], c["ll"], m_ac = _middle(a["ll"], c["ll"])
        b["ll"], c["ll"], m_bc = _middle(b["ll"], c["ll"])
        return {"ll": m_ab, "sn": ab}, {"ll": m_ac, "sn": ac}, {"ll": m_bc, "sn": bc}

    def bisect(self, a, b, c, level):
        """bisect_triangle_nasr (bisect_triangle.F90:134-191)."""
        clevel = level + 1
        self._store(a, b, c)
        if clevel > self.ml:
            return
        ab, ac, bc = self._split(a, b, c, clevel, 1)
        self.bisect(a, ab, ac, clevel)
        self.bisect(ab, b, bc, clevel)
        self.bisect_r(ab, ac, bc, clevel)
        self.bisect(ac, bc, c, clevel)

    def bisect_r(self, a, b, c, level):
        """bisect_r_triangle_nasr (bisect_triangle.F90:194-253)."""
        self._store(a, b, c)
        clevel = level + 1
        if clevel > self.ml:
            return
        ab, ac, bc = self._split(a, b, c, clevel, 0)
        self.bisect_r(a, ab, ac, clevel)
        self.bisect(ab, ac, bc, clevel)
        self.bisect_r(ab, b, bc, clevel)
        self.bisect_r(ac, bc, c, clevel)

    def remove_edge1(self, t):
        sl = self.sl
        stride, idx = sl + 1, t["start"]
        while idx <= t["end"] and stride >= 0:
            self.seq[idx] = -1
            idx += stride
            stride -= 1
        self._compact(t)

    def remove_edge2(self, t):
        sl = self.sl
        for idx in range(t["start"], t["start"] + sl + 1):
            self.seq[idx] = -1
        stride, idx = sl - 1, t["start"] + sl * 2
        while idx <= t["end"] and stride >= 0:
            self.seq[idx] = -1
            idx += stride
            stride -= 1
        self._compact(t)

    def _compact(self, t):
        stride, idx2 = 0, t["start"]
        for idx in range(t["start"], t["end"] + 1):
            if self.seq[idx] == -1:
                stride += 1
                continue
            self.lat[idx2], self.lon[idx2] = self.lat[idx], self.lon[idx]
            self.seq[idx2] = self.seq[idx] - stride
            idx2 += 1
        t["end"] -= stride

    def combine(self, t1, t2):
        sl = self.sl
        last = self.seq[t2["end"]]
        for idx in range(t2["start"], t2["end"] + 1):
            self.seq[idx] = last - self.seq[idx]
        stride, gap, delta = sl - 3, 1, 1
        idx = t1["start"] + (2 * sl - 1)
        while idx <= t1["end"]:
            idx2 = idx
            for idx2 in range(idx, idx + stride + 1):
                self.seq[idx2] += gap
            idx2 = idx + stride + 1  # the DO variable's value after the loop
            stride -= 1
            delta += 1
            gap += delta
            idx = idx2
        stride, gap, delta = 0, 2 * sl - 1, sl - 1
        idx = t2["end"]
        while idx >= t2["start"]:
            for idx2 in range(idx, idx - stride - 1, -1):
                self.seq[idx2] += gap
            idx2 = idx - stride - 1
            stride += 1
            delta -= 1
            gap += delta
            idx = idx2

    def run(self):
        sl = self.sl
        top = _top_grid()
        tri = _top_triangles(top)
        ts = [None] * 21
        for i in range(1, 21):
            self.offset = (i - 1) * (self.init_c_sn + 1) + 1
            v = [{"ll": list(tri[i][0]), "sn": 0}, {"ll": list(tri[i][1]), "sn": sl},
                 {"ll": list(tri[i][2]), "sn": self.init_c_sn}]
            ts[i] = {"start": self.offset, "end": self.offset + self.init_c_sn}
            self.bisect(v[0], v[1], v[2], 0)
        for i in list(range(1, 6)) + list(range(11, 16)):
            self.remove_edge1(ts[i])
        for i in list(range(6, 11)) + list(range(16, 21)):
            self.remove_edge2(ts[i])
        for i in range(1, 6):
            self.combine(ts[i], ts[i + 15])
        for i in range(6, 10):
            self.combine(ts[i + 6], ts[i])
        self.combine(ts[11], ts[10])
        off = sl * sl

        def shift(t, d):
            for k in range(t["start"], t["end"] + 1):
                self.seq[k] += d

        for j in range(1, 6):
            shift(ts[j], (j - 1) * off * 2 + 1)
        for j in range(16, 21):
            shift(ts[j], (j - 16) * off * 2 + 1)
        for j in range(12, 16):
            shift(ts[j], (j - 12) * off * 2 + off + 1)
        shift(ts[11], 4 * off * 2 + off + 1)
        for j in range(6, 11):
            shift(ts[j], (j - 6) * off * 2 + off + 1)
        nip = 10 * sl * sl + 2
        lat = np.full(nip + 1, np.nan)
        lon = np.full(nip + 1, np.nan)
        lat[1], lon[1] = top[1]["ll"]
        lat[nip], lon[nip] = top[7]["ll"]
        for j in range(1, 21):
            for k in range(ts[j]["start"], ts[j]["end"] + 1):
                s = self.seq[k] + 1
                if not np.isnan(lat[s]):
                    raise AssertionError("sequence number %d written twice" % s)
                lat[s], lon[s] = self.lat[k], self.lon[k]
        return lat[1:], lon[1:]


def icos_points(glvl):
    """(lat, lon) in degrees of grid points 1..nip in the reference's order
    (icos_grid_level.dat of icos.F90:100-119)."""
    return _Icos(glvl).run()


def _grid_point_type(seq, diam, el):
    """GridGen.F90:503-526."""
    i = (seq - 1) % (2 * diam)
    if i < el:
        return 1
    if i % el == 0 and i <= diam:
        return 2
    if i % el == 0 and i < 2 * diam:
        return 3
    if i % el == 1 and i < diam:
        return 4
    if i % el == 1 and i < 2 * diam:
        return 5
    if i >= 2 * diam - el + 1:
        return 6
    return 0


def _special_points(i, diam, el):
    """GridGen.F90:529-623: (nb, type) for the poles, rhombus corners and
    pentagons; type 0 leaves nb unset."""
    nb = [0] * 6
    r_i = (i - 1) % (2 * diam)
    if i == 1:
        nb[0] = 2
        for k in range(1, 5):
            nb[k] = nb[k - 1] + 2 * diam
        nb[5] = -1
        return nb, 1
    if i == 10 * diam + 2:
        nb[0] = 10 * diam + 1
        for k in range(1, 5):
            nb[k] = nb[k - 1] - 2 * diam
        nb[5] = -1
        return nb, 1
    if r_i == 1:
        nb[0] = 1
        nb[1] = i - 2 * diam if i - 2 * diam > 0 else i + 8 * diam
        nb[2] = nb[1] + el
        nb[3] = i + 1
        nb[4] = i + el
        nb[5] = (i + 2 * diam) % (10 * diam)
        return nb, 2
    if r_i == 0:
        nb[0] = i - el
        nb[1] = i - 2 * diam - 1 if i - 4 * diam > 0 else i + 8 * diam - 1
        nb[2] = nb[1] + 1
        nb[3] = 10 * diam + 2
        nb[4] = i + 2 * diam if i + 2 * diam <= 10 * diam + 1 else i + 2 * diam - 10 * diam
        nb[5] = i - 1
        return nb, 2
    if r_i == el:
        nb[0] = i - 1
        pg = i // (2 * diam)
        pg = pg - 1 if pg >= 1 else 4
        nb[1] = pg * 2 * diam + diam - el + 2
        nb[2] = nb[1] + el
        nb[3] = i + el
        nb[4] = nb[3] - 1
        nb[5] = -1
        return nb, 1
    if r_i == diam + el:
        nb[0] = i - 1
        nb[1] = i - el
        pg = i // (2 * diam)
        pg = pg - 1 if pg >= 1 else 4
        nb[2] = pg * 2 * diam + 2 * diam - el + 2
        nb[3] = i + el
        nb[4] = nb[3] - 1
        nb[5] = -1
        return nb, 1
    if r_i == 2 * diam - el + 1:
        nb[0] = i - el
        nb[1] = nb[0] + 1
        nb[2] = nb[1] + el
        pg = (i - 1) // (2 * diam)
        pg = pg + 1 if pg < 4 else 0
        r2 = (i - 1) % (2 * diam)
        nb[3] = pg * 2 * diam + r2 - diam + 3 * el
        nb[4] = nb[3] - el
        nb[5] = nb[4] - el
        return nb, 2
    return nb, 0


def _pattern_neighbours(i, diam, el):
    """GridGen.F90:117-210 for an ordinary point (special_points type 0)."""
    gp_type = _grid_point_type(i, diam, el)
    nb = [0] * 6
    pg_up = (i - 1) // (2 * diam)
    pg_prev = pg_up - 1 if pg_up >= 1 else 4
    pg_next = pg_up + 1 if pg_up < 4 else 0
    r_i = (i - 1) % (2 * diam)
    if gp_type == 0:
        nb = [i - 1, i - el, i - el + 1, i + 1, i + el, i + el - 1]
    elif gp_type == 1:
        nb[0] = i - 1
        nb[1] = pg_prev * 2 * diam + (r_i - 1) * el + 2
        nb[2] = nb[1] + el
        nb[3] = i + 1
        nb[4] = i + el
        nb[5] = i + el - 1
    elif gp_type == 2:
        nb[0] = i - el
        nb[1] = pg_prev * 2 * diam + diam - 2 * el + r_i + 2
        nb[2] = nb[1] + el
        nb[3] = i + el
        nb[4] = nb[3] - 1
        nb[5] = i - 1
    elif gp_type == 3:
        nb[0] = i - el
        nb[1] = (pg_prev + 1) * 2 * diam - el + (r_i - (diam + 2 * el)) // el + 2
        nb[2] = nb[1] + 1
        nb[3] = i + el
        nb[4] = nb[3] - 1
        nb[5] = i - 1
    elif gp_type == 4:
        nb[0] = i - el
        nb[1] = nb[0] + 1
        nb[2] = i + 1
        nb[3] = i + el
        nb[4] = pg_next * 2 * diam + 2 + (r_i - 1) // el
        nb[5] = nb[4] - 1
    elif gp_type == 5:
        nb[0] = i - el
        nb[1] = nb[0] + 1
        nb[2] = nb[1] + el
        nb[3] = i + el
        nb[4] = pg_next * 2 * diam + r_i - diam + 2 * el
        nb[5] = nb[4] - el
    elif gp_type == 6:
        nb[0] = i - 1
        nb[1] = i - el
        nb[2] = nb[1] + 1
        nb[3] = i + 1
        nb[4] = pg_next * 2 * diam + diam + (r_i - 2 * diam + el + 1) * el + 1
        nb[5] = nb[4] - el
    return nb


def neighbour_tables(glvl):
    """(nprox, prox, proxs) as the reference's dycore holds them after
    dyn_init: 1-based, prox/proxs of shape (nip, 6) (slot fastest), a
    pentagon's prox slot 6 repeating slot 5 and its proxs slot 6 = -99."""
    sl = 2 ** glvl
    nip = 10 * sl * sl + 2
    diam = (nip - 2) // 10
    el = int(math.sqrt(float(diam)) + 0.5)
    prox = np.zeros((nip + 1, 6), np.int64)
    nprox = np.full(nip + 1, 6, np.int64)
    for i in range(1, nip + 1):
        nb, sgp = _special_points(i, diam, el)
        if sgp == 1:
            nprox[i] = 5
        if sgp == 0:
            nb = _pattern_neighbours(i, diam, el)
        prox[i] = nb
    # getlvl.F90:145-157
    proxs = np.full((nip + 1, 6), -99, np.int64)
    for ipn in range(1, nip + 1):
        for isn in range(nprox[ipn]):
            ip = prox[ipn, isn]
            for j in range(nprox[ip]):
                if prox[ip, j] == ipn:
                    proxs[ipn, isn] = j + 1
                    break
    # dyn_init.F90:545-549
    pent = nprox == 5
    prox[pent, 5] = prox[pent, 4]
    return nprox[1:], prox[1:], proxs[1:]
