"""Reader and writer of FIM's grid file glvl.dat.

The file is a Fortran unformatted sequential file (4-byte record markers)
written by FIMsrc/prep/grid/getlvl.F90:296-346 and read by
FIMsrc/fim/horizontal/dyn_init.F90:373-541: two 16-character header records
("glvl =NN", "curve =NN", FIMsrc/utils/headers.F90:10-26), then lat, lon,
nprox, proxs(6 records), prox(6), area, cs(4x6), sn(4x6), sidevec_c(2x6),
sidevec_e(2x6), sideln(6), rprox_ln(6), inv_perm, corner_xy(6x2) and
hfcoef(6x6), one record per (component, edge) pair, each of nip real*4 or
integer*4 values.  With this reader a grid produced by the reference's own
generator (any curve / gtype) can be handed to fim_ctx_create.
"""
import struct

import numpy as np

_I4 = np.dtype("<i4")
_R4 = np.dtype("<f4")


def _write_rec(fh, data: bytes):
    fh.write(struct.pack("<i", len(data)))
    fh.write(data)
    fh.write(struct.pack("<i", len(data)))


def _read_rec(fh):
    head = fh.read(4)
    if len(head) < 4:
        raise EOFError("glvl.dat ended early")
    (n,) = struct.unpack("<i", head)
    data = fh.read(n)
    (tail,) = struct.unpack("<i", fh.read(4))
    if tail != n or len(data) != n:
        raise ValueError("corrupt Fortran record (%d vs %d)" % (n, tail))
    return data


class GridTables:
    """Grid tables in the layout of Grid (reference layout, 1-based numbers)."""

    def __init__(self, glvl, nip):
        self.glvl = glvl
        self.nip = nip

    def desc(self):
        from .grid import Grid
        return Grid.desc(self)

    def zero_based(self):
        from .grid import Grid
        return Grid.zero_based(self)


def write_glvl_dat(grid, path, curve=0):
    """Write `grid` in the reference's glvl.dat layout (real*4 tables)."""
    nip = grid.nip
    f = lambda a: np.ascontiguousarray(a, dtype=_R4).tobytes()  # noqa: E731
    i = lambda a: np.ascontiguousarray(a, dtype=_I4).tobytes()  # noqa: E731
    prox = grid.prox.reshape(nip, 6)
    proxs = grid.proxs.reshape(nip, 6)
    with open(path, "wb") as fh:
        _write_rec(fh, ("glvl =%2d" % grid.glvl).ljust(16).encode())
        _write_rec(fh, ("curve =%2d" % curve).ljust(16).encode())
        _write_rec(fh, f(grid.lat))
        _write_rec(fh, f(grid.lon))
        _write_rec(fh, i(grid.nprox))
        for isn in range(6):
            _write_rec(fh, i(proxs[:, isn]))
        for isn in range(6):
            _write_rec(fh, i(prox[:, isn]))
        _write_rec(fh, f(grid.area))
        for name, ncomp in (("cs", 4), ("sn", 4), ("sidevec_c", 2), ("sidevec_e", 2)):
            a = getattr(grid, name).reshape(nip, 6, ncomp)
            for isn in range(6):
                for idx in range(ncomp):
                    _write_rec(fh, f(a[:, isn, idx]))
        for name in ("sideln", "rprox_ln"):
            a = getattr(grid, name).reshape(nip, 6)
            for isn in range(6):
                _write_rec(fh, f(a[:, isn]))
        _write_rec(fh, i(np.arange(1, nip + 1)))  # inv_perm: identity for the IJ order
        cxy = grid.corner_xy.reshape(nip, 2, 6)
        for ixy in range(2):
            for isn in range(6):
                _write_rec(fh, f(cxy[:, ixy, isn]))
        hf = grid.hfcoef.reshape(nip, 6, 6)
        for isn in range(6):
            for idx in range(6):
                _write_rec(fh, f(hf[:, isn, idx]))


def read_glvl_dat(path, glvl=None):
    """Read glvl.dat into GridTables (float64 copies of the real*4 tables).

    Pentagons get prox(6) = prox(5) as dyn_init.F90:545-549 does; the file's
    permutation (inv_perm) is returned as .perm for callers that reorder
    their own fields; the tables themselves are in file order.
    """
    with open(path, "rb") as fh:
        h1 = _read_rec(fh).decode(errors="replace")
        h2 = _read_rec(fh).decode(errors="replace")
        g = int(h1[6:8])
        if glvl is not None and glvl != g:
            raise ValueError("glvl.dat header says glvl=%d, expected %d" % (g, glvl))
        lat = np.frombuffer(_read_rec(fh), _R4).astype(np.float64)
        nip = lat.size
        t = GridTables(g, nip)
        t.curve = int(h2[7:9])
        t.lat = lat
        t.lon = np.frombuffer(_read_rec(fh), _R4).astype(np.float64)
        t.nprox = np.frombuffer(_read_rec(fh), _I4).astype(np.int32)
        proxs = np.stack([np.frombuffer(_read_rec(fh), _I4) for _ in range(6)], 1)
        prox = np.stack([np.frombuffer(_read_rec(fh), _I4) for _ in range(6)], 1).copy()
        pent = t.nprox == 5
        prox[pent, 5] = prox[pent, 4]
        t.proxs = proxs.astype(np.int32).reshape(-1)
        t.prox = prox.astype(np.int32).reshape(-1)
        t.area = np.frombuffer(_read_rec(fh), _R4).astype(np.float64)
        for name, ncomp in (("cs", 4), ("sn", 4), ("sidevec_c", 2), ("sidevec_e", 2)):
            a = np.zeros((nip, 6, ncomp))
            for isn in range(6):
                for idx in range(ncomp):
                    a[:, isn, idx] = np.frombuffer(_read_rec(fh), _R4)
            setattr(t, name, a.reshape(-1))
        for name in ("sideln", "rprox_ln"):
            a = np.zeros((nip, 6))
            for isn in range(6):
                a[:, isn] = np.frombuffer(_read_rec(fh), _R4)
            setattr(t, name, a.reshape(-1))
        t.perm = np.frombuffer(_read_rec(fh), _I4).astype(np.int32)
        cxy = np.zeros((nip, 2, 6))
        for ixy in range(2):
            for isn in range(6):
                cxy[:, ixy, isn] = np.frombuffer(_read_rec(fh), _R4)
        t.corner_xy = cxy.reshape(-1)
        hf = np.zeros((nip, 6, 6))
        for isn in range(6):
            for idx in range(6):
                hf[:, isn, idx] = np.frombuffer(_read_rec(fh), _R4)
        t.hfcoef = hf.reshape(-1)
    for n in ("lat", "lon", "area", "cs", "sn", "sidevec_c", "sidevec_e", "sideln", "rprox_ln", "corner_xy",
              "hfcoef"):
        setattr(t, n, np.ascontiguousarray(getattr(t, n), np.float64))
    return t
