"""The C-ABI library loads and exports every entry point of include/fim_gpu.h."""
import os
import re

import fimocn_subx_realtime_hera_apr2020_gb300._lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "fim_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fim_\w+)\s*\(", src)))


def test_library_exports_header_symbols():
    lib = L.load()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(header_functions()) == set(L.EXPORTED)


def test_grid_nip():
    lib = L.load()
    assert [lib.fim_grid_nip(g) for g in (4, 6, 7, 8)] == [2562, 40962, 163842, 655362]
    assert lib.fim_grid_nip(-1) == -1


def test_ctx_rejects_edge_without_mirror():
    """fim_ctx_create checks prox(proxs(e,i), prox(e,i)) == i for every edge
    before it touches the device, so a broken table fails with FIM_EINVAL."""
    import numpy as np
    import pytest
    import fimocn_subx_realtime_hera_apr2020_gb300 as F
    g = F.Grid(4)
    ps = g.proxs.reshape(-1, 6)
    i = 100
    ps[i, 0] = ps[i, 0] % 6 + 1  # point edge 0 of cell 100 at the wrong mirror slot
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0, precision="f64")
    with pytest.raises(L.FimError) as err:
        F.Dycore(g, cfg)
    assert err.value.code == L.FIM_EINVAL
    assert np.all(ps[:, :5] >= 1)


def test_ctx_rejects_bad_configurations():
    """Configuration checks of fim_ctx_create run before any device call."""
    import pytest
    import fimocn_subx_realtime_hera_apr2020_gb300 as F
    g = F.Grid(4)
    base = dict(nvl=38, ntra=5, dt=400.0, precision="f64")
    cases = [
        (dict(base, ntra=3), L.FIM_EINVAL),                    # theta + at least 3 tracers
        (dict(base, flux_conserv_schm=3), L.FIM_ENOTSUP),
        (dict(base, pure_sig=1), L.FIM_ENOTSUP),
        (dict(base, remap_optn=4), L.FIM_EINVAL),
        (dict(base, ntrb=-1), L.FIM_EINVAL),
        (dict(base, ntra=20, ntrb=13), L.FIM_EINVAL),          # ntra + ntrb <= 32
        (dict(base, dt=0.0), L.FIM_EINVAL),
    ]
    for kw, code in cases:
        with pytest.raises(L.FimError) as err:
            F.Dycore(g, F.FimConfig(**kw))
        assert err.value.code == code, kw
    # edgvar2 in the step needs the grid's corner_xy table
    g2 = F.Grid(4)
    g2.corner_xy = None
    with pytest.raises(L.FimError) as err:
        F.Dycore(g2, F.FimConfig(**dict(base, hi_order_uv_comp=1)))
    assert err.value.code == L.FIM_EINVAL
