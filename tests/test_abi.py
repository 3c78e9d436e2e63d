"""The C-ABI library loads and exports every symbol include/*.h declares (no
GPU needed: no compute call is made), and argument validation happens on
the host before any device work."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ss_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported_and_bound():
    from superscanner_gb300 import _native
    declared = _declared()
    assert len(declared) >= 15, declared
    for name in declared:
        assert hasattr(_native.lib, name), name
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"
    assert set(_native.SIGNATURES) <= declared


def test_host_side_argument_errors():
    from superscanner_gb300 import _native as n
    lib = n.lib
    p = n.SSParams()
    assert lib.ss_params_default(None, 1 << 20, 0.02, 0.005, 480, 640) == n.SS_ERR_ARG
    assert lib.ss_params_default(C.byref(p), 1 << 20, -1.0, 0.005, 480, 640) == n.SS_ERR_ARG
    assert lib.ss_params_default(C.byref(p), int(1e8), 0.05, 0.01, 480, 640) == n.SS_OK
    assert p.hash_buckets == 1 << 18 and p.rmin == pytest.approx(0.2) and p.d_max == pytest.approx(10.0)
    bad = n.SSParams.from_buffer_copy(p)
    bad.hash_buckets = 1000  # not a power of two
    h = C.c_void_p()
    assert lib.ss_grid_create(C.byref(bad), C.byref(h)) == n.SS_ERR_ARG
    assert lib.ss_grid_create(None, C.byref(h)) == n.SS_ERR_ARG
    assert lib.ss_grid_destroy(None) == n.SS_ERR_ARG
    assert lib.ss_integrate(None, None, None, None, 0, None) == n.SS_ERR_ARG
    assert lib.ss_raycast(None, None, None, None, None) == n.SS_ERR_ARG
    out = (C.c_double * 16)()
    assert lib.ss_kokkos_icp(None, None, 480, 640, 525.0, 525.0, 319.5, 239.5, None, None, 0, out, None,
                             None) == n.SS_ERR_ARG
