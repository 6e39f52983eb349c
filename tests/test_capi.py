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
