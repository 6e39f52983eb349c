"""Icosahedral-hexagonal grid tables (host side).

Wraps fim_grid_build of the C-ABI, which restates the reference grid chain
(FIMsrc/prep/grid/icos.F90 -> GridGen.F90 -> getlvl.F90).  Tables keep the
reference layout and Fortran (1-based) numbering, exactly what a caller
holding glvl.dat would pass to fim_ctx_create (dyn_init.F90:373-549).
"""
import ctypes

import numpy as np

from . import _lib

_CACHE = {}


class Grid:
    """Grid tables of one icosahedral level, as numpy arrays."""

    NAMES_I = ("nprox", "prox", "proxs")
    NAMES_D = ("lat", "lon", "area", "cs", "sn", "sidevec_c", "sidevec_e", "sideln", "rprox_ln",
               "corner_xy", "hfcoef")

    def __init__(self, glvl):
        lib = _lib.load()
        nip = lib.fim_grid_nip(glvl)
        if nip <= 0:
            raise ValueError("unsupported grid level %d" % glvl)
        self.glvl = glvl
        self.nip = nip
        sizes = dict(nprox=nip, prox=6 * nip, proxs=6 * nip, lat=nip, lon=nip, area=nip, cs=24 * nip,
                     sn=24 * nip, sidevec_c=12 * nip, sidevec_e=12 * nip, sideln=6 * nip, rprox_ln=6 * nip,
                     corner_xy=12 * nip, hfcoef=36 * nip)
        for n in self.NAMES_I:
            setattr(self, n, np.zeros(sizes[n], np.int32))
        for n in self.NAMES_D:
            setattr(self, n, np.zeros(sizes[n], np.float64))
        desc = self.desc()
        _lib.check(lib.fim_grid_build(glvl, ctypes.byref(desc)), "fim_grid_build")

    @classmethod
    def cached(cls, glvl):
        if glvl not in _CACHE:
            _CACHE[glvl] = cls(glvl)
        return _CACHE[glvl]

    def desc(self):
        d = _lib.GridDesc()
        d.glvl = self.glvl
        d.nip = self.nip
        for n in self.NAMES_I + self.NAMES_D:
            a = getattr(self, n)
            setattr(d, n, a.ctypes.data if a is not None else None)  # optional tables may be absent
        return d

    def zero_based(self):
        """0-based neighbour tables (the CPU oracle's convention)."""
        nprox = self.nprox.astype(np.int32)
        prox = (self.prox - 1).astype(np.int32)
        proxs = np.where(self.proxs > 0, self.proxs - 1, -1).astype(np.int32)
        return nprox, prox, proxs
