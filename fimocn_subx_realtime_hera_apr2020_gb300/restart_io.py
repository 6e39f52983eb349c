"""Restart files of the dynamics state in the reference's layout.

A FIM restart file (FIMsrc/fim/horizontal/restart.F90:40-60) is a Fortran
unformatted sequential file (4-byte record markers): one record with itsm1,
the completed step count, then the dynamics section that write_restart_dyn
writes (restart_dyn.F90:94-168), then the coupler, physics and ocean
sections.  The dynamics section is

  1  curr_write_time, nf, of, vof, adbash1..3, thetac(nvl), dpsig(nvl),
     sigak(nvlsig+1), sigbk(nvlsig+1)
  2  lat, lon, nprox, proxs(6,nip), area, cs(4,6,nip), sn(4,6,nip), psrf,
     ptdcy(nip,2)
  3  qmstr, qmstrc, qmstrn, qdtr_set
  4  sidevec_c(2,6,nip), sidevec_e(2,6,nip), sideln(6,nip), rprox_ln(6,nip)
  5  sst_prev, sst_next, fice2d_prev, fice2d_next, fice2d, next_date(4),
     have_next_sst
  6  rarea, rsideln(6,nip), corio, deg_lat, deg_lon, rn2d, pw2d, rc2d, u10m,
     v10m, runoff

followed by one 32-bit record per (level[, edge]) x nip array slice: the AB3
tendency slots of u, v, dp, dp_lo; per tracer tr3d, trdp and its trc/trl
tendency slots; us3d, vs3d, ws3d, mp3d, tk3d, dp3d, rh3d, relvor, dpinit;
pr3d, ex3d, ph3d, sdot; the three massfx slots and cumufx.  Integers and
logicals are 4 bytes; the scalar records' reals have the build's default
kind (4 bytes for FIM's -r4 dynamics, `real_bytes`), the array records are
always real*4 (readarr32_r.F90, writearr32_r.F90).

Fields that belong to the physics (sst, ice, rain, tk3d, rh3d, ...) are
written as zeros unless given in `extras`, and returned in `extras` when
read.  Class-B tracers (cfg.ntrb) follow the class-A ones; their AB3
tendency records, which the class-B transport does not use, are zeros.
Only the dynamics section is written; reading stops after it, so a full
reference restart file is read.

Between fim_step calls the library state is the reference's state between
dyn_run calls, so a restart file written here resumes the same forecast
in either code, to the precision of the file's 32-bit records.
"""
import struct

import numpy as np

_I4 = np.dtype("<i4")
_R4 = np.dtype("<f4")

# dynamics fields of the library state that the restart file carries
STATE_FIELDS = ["u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy", "tr3d", "trdp", "trc_tdcy", "trl_tdcy", "us3d",
                "vs3d", "ws3d", "mp3d", "dp3d", "relvor", "pr3d", "ex3d", "ph3d", "sdot", "massfx", "psrf", "ptdcy",
                "dpinit", "cumufx"]
_SFC = ["sst_prev", "sst_next", "fice2d_prev", "fice2d_next", "fice2d"]
_REC6 = ["rn2d", "pw2d", "rc2d", "u10m", "v10m", "runoff"]
_CELL_EXTRA = ["tk3d", "rh3d"]


def _rec(fh, *parts):
    data = b"".join(parts)
    fh.write(struct.pack("<i", len(data)))
    fh.write(data)
    fh.write(struct.pack("<i", len(data)))


def _read_rec(fh):
    head = fh.read(4)
    if len(head) < 4:
        raise EOFError("restart file ended early")
    (n,) = struct.unpack("<i", head)
    data = fh.read(n)
    tail = fh.read(4)
    if len(data) != n or len(tail) != 4 or struct.unpack("<i", tail)[0] != n:
        raise ValueError("corrupt Fortran record (length %d)" % n)
    return data


class _Cursor:
    def __init__(self, data):
        self.data = data
        self.pos = 0

    def take(self, dtype, count):
        dt = np.dtype(dtype)
        end = self.pos + dt.itemsize * count
        if end > len(self.data):
            raise ValueError("record shorter than the layout expects")
        out = np.frombuffer(self.data[self.pos:end], dt).copy()
        self.pos = end
        return out

    def done(self):
        if self.pos != len(self.data):
            raise ValueError("record longer than the layout expects (%d of %d bytes read)" %
                             (self.pos, len(self.data)))


def _f(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype).tobytes()


def write_restart(path, grid, cfg, itsm1, nf, of, vof, adbash, fields, extras=None, nvlsig=None, real_bytes=4):
    """Write the dynamics section of a restart file.

    `fields`: flat arrays in the library / reference layout (STATE_FIELDS;
    tr3d and trdp for ntra + ntrb tracers, the tendencies for ntra).  nf/of/vof
    are in Fortran numbering; adbash = (adbash1, adbash2, adbash3).
    """
    nip, nvl = grid.nip, cfg.nvl
    nta = cfg.ntra
    ntra = nta + getattr(cfg, "ntrb", 0)
    nvlsig = nvl if nvlsig is None else nvlsig
    ex = dict(extras or {})
    rdt = np.dtype("<f%d" % real_bytes)
    z = lambda n: np.zeros(n)  # noqa: E731
    get = lambda k, n: np.asarray(ex.get(k, z(n)), np.float64).reshape(-1)  # noqa: E731
    lat = np.asarray(grid.lat, np.float64)
    with open(path, "wb") as fh:
        _rec(fh, _f([itsm1], _I4))
        _rec(fh, _f([ex.get("curr_write_time", 0), nf, of, vof], _I4), _f(adbash, rdt), _f(cfg.thetac, rdt),
             _f(cfg.dpsig, rdt), _f(get("sigak", nvlsig + 1), rdt), _f(get("sigbk", nvlsig + 1), rdt))
        _rec(fh, _f(lat, rdt), _f(grid.lon, rdt), _f(grid.nprox, _I4), _f(grid.proxs, _I4), _f(grid.area, rdt),
             _f(grid.cs, rdt), _f(grid.sn, rdt), _f(fields["psrf"], rdt), _f(fields["ptdcy"], rdt))
        _rec(fh, _f([get("qmstr", 1)[0], get("qmstrc", 1)[0], get("qmstrn", 1)[0]], rdt),
             _f([1 if ex.get("qdtr_set", False) else 0], _I4))
        _rec(fh, _f(grid.sidevec_c, rdt), _f(grid.sidevec_e, rdt), _f(grid.sideln, rdt), _f(grid.rprox_ln, rdt))
        _rec(fh, *[_f(get(k, nip), rdt) for k in _SFC],
             _f(np.asarray(ex.get("next_date", [0, 0, 0, 0])), _I4), _f([1 if ex.get("have_next_sst") else 0], _I4))
        sideln = np.asarray(grid.sideln, np.float64)
        rsideln = np.divide(1.0, sideln, out=np.zeros_like(sideln), where=sideln != 0)
        _rec(fh, _f(1.0 / np.asarray(grid.area, np.float64), rdt), _f(rsideln, rdt),
             _f(1.4584e-4 * np.sin(lat), rdt), _f(np.degrees(lat), rdt), _f(np.degrees(grid.lon), rdt),
             *[_f(get(k, nip), rdt) for k in _REC6])
        cell = nvl * nip
        slab = lambda name, j, n=cell: _f(np.asarray(fields[name]).reshape(-1)[j * n:(j + 1) * n], _R4)  # noqa: E731
        for n in range(3):
            for name in ("u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy"):
                _rec(fh, slab(name, n))
        for t in range(ntra):
            _rec(fh, slab("tr3d", t))
            _rec(fh, slab("trdp", t))
            for n in range(3):
                for name in ("trc_tdcy", "trl_tdcy"):
                    _rec(fh, slab(name, t * 3 + n) if t < nta else _f(z(cell), _R4))
        def part(name, n):
            a = np.asarray(fields[name] if name in fields else ex.get(name, z(n))).reshape(-1)
            return _f(a[:n] if a.size else z(n), _R4)

        for name in ("us3d", "vs3d", "ws3d", "mp3d", "tk3d", "dp3d", "rh3d", "relvor", "dpinit"):
            _rec(fh, part(name, cell))
        for name in ("pr3d", "ex3d", "ph3d", "sdot"):
            _rec(fh, slab(name, 0, (nvl + 1) * nip))
        for n in range(3):
            _rec(fh, slab("massfx", n, 6 * cell))
        _rec(fh, part("cumufx", 6 * cell))


def read_restart(path, nip, nvl, ntra, ntrb=0, nvlsig=None, real_bytes=4):
    """Read itsm1 and the dynamics section; returns a dict with itsm1, nf,
    of, vof (Fortran numbering), adbash, fields (STATE_FIELDS, float32 flat
    arrays in the library layout) and extras (everything else)."""
    nvlsig = nvl if nvlsig is None else nvlsig
    rdt = np.dtype("<f%d" % real_bytes)
    nt = ntra + ntrb
    cell = nvl * nip
    fields, extras = {}, {}
    with open(path, "rb") as fh:
        c = _Cursor(_read_rec(fh))
        itsm1 = int(c.take(_I4, 1)[0])
        c.done()
        c = _Cursor(_read_rec(fh))
        cw, nf, of, vof = (int(x) for x in c.take(_I4, 4))
        adbash = tuple(float(x) for x in c.take(rdt, 3))
        extras["curr_write_time"] = cw
        extras["thetac"] = c.take(rdt, nvl)
        extras["dpsig"] = c.take(rdt, nvl)
        extras["sigak"] = c.take(rdt, nvlsig + 1)
        extras["sigbk"] = c.take(rdt, nvlsig + 1)
        c.done()
        c = _Cursor(_read_rec(fh))
        extras["lat"] = c.take(rdt, nip)
        extras["lon"] = c.take(rdt, nip)
        extras["nprox"] = c.take(_I4, nip)
        extras["proxs"] = c.take(_I4, 6 * nip)
        extras["area"] = c.take(rdt, nip)
        extras["cs"] = c.take(rdt, 24 * nip)
        extras["sn"] = c.take(rdt, 24 * nip)
        fields["psrf"] = c.take(rdt, nip).astype(np.float32)
        fields["ptdcy"] = c.take(rdt, 2 * nip).astype(np.float32)
        c.done()
        c = _Cursor(_read_rec(fh))
        extras["qmstr"], extras["qmstrc"], extras["qmstrn"] = (float(x) for x in c.take(rdt, 3))
        extras["qdtr_set"] = bool(c.take(_I4, 1)[0])
        c.done()
        c = _Cursor(_read_rec(fh))
        for name, n in (("sidevec_c", 12 * nip), ("sidevec_e", 12 * nip), ("sideln", 6 * nip),
                        ("rprox_ln", 6 * nip)):
            extras[name] = c.take(rdt, n)
        c.done()
        c = _Cursor(_read_rec(fh))
        for name in _SFC:
            extras[name] = c.take(rdt, nip)
        extras["next_date"] = c.take(_I4, 4)
        extras["have_next_sst"] = bool(c.take(_I4, 1)[0])
        c.done()
        c = _Cursor(_read_rec(fh))
        extras["rarea"] = c.take(rdt, nip)
        extras["rsideln"] = c.take(rdt, 6 * nip)
        for name in ("corio", "deg_lat", "deg_lon") + tuple(_REC6):
            extras[name] = c.take(rdt, nip)
        c.done()

        def arr(n):
            c = _Cursor(_read_rec(fh))
            a = c.take(_R4, n)
            c.done()
            return a

        slots = {k: [None] * 3 for k in ("u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy")}
        for n in range(3):
            for name in ("u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy"):
                slots[name][n] = arr(cell)
        for name, parts in slots.items():
            fields[name] = np.concatenate(parts)
        tr, td, tc, tl = [], [], [], []
        for t in range(nt):
            tr.append(arr(cell))
            td.append(arr(cell))
            for n in range(3):
                a, b = arr(cell), arr(cell)
                if t < ntra:  # class-B tendency records carry nothing the transport uses
                    tc.append(a)
                    tl.append(b)
        fields["tr3d"], fields["trdp"] = np.concatenate(tr), np.concatenate(td)
        fields["trc_tdcy"], fields["trl_tdcy"] = np.concatenate(tc), np.concatenate(tl)
        for name in ("us3d", "vs3d", "ws3d", "mp3d", "tk3d", "dp3d", "rh3d", "relvor", "dpinit"):
            (fields if name in STATE_FIELDS else extras)[name] = arr(cell)
        for name in ("pr3d", "ex3d", "ph3d", "sdot"):
            fields[name] = arr((nvl + 1) * nip)
        fields["massfx"] = np.concatenate([arr(6 * cell) for _ in range(3)])
        fields["cumufx"] = arr(6 * cell)
    return {"itsm1": itsm1, "nf": nf, "of": of, "vof": vof, "adbash": adbash, "fields": fields, "extras": extras}
