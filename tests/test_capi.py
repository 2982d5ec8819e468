"""Host-side checks of the C-ABI library (no GPU needed): it builds, loads,
exports every entry point include/aeros_gpu.h declares, and its host-only
entry points (grid sizing, parameter defaults) give the reference's values."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "aeros_gpu.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(aeros_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from aeros_gb300 import build
    build.build()
    from aeros_gb300 import _capi
    return _capi.lib()


def test_every_declared_symbol_is_exported(lib):
    from aeros_gb300 import _capi
    names = declared_symbols()
    assert len(names) >= 40
    for n in names:
        assert hasattr(lib, n), n
        assert n in _capi._PROTOS, f"{n} has no ctypes prototype"


def test_grid_size_host_only(lib):
    a, b = ctypes.c_int(), ctypes.c_int()
    for T, grid in [(21, (64, 32)), (31, (96, 48)), (42, (128, 64)), (85, (256, 128)), (341, (1024, 512))]:
        assert lib.aeros_sht_grid_size(T, ctypes.byref(a), ctypes.byref(b)) == 0
        assert (a.value, b.value) == grid
    assert lib.aeros_sht_grid_size(0, ctypes.byref(a), ctypes.byref(b)) == -1


def test_params_default_is_held_suarez(lib):
    from aeros_gb300.params import AerosParams, held_suarez_params
    p = AerosParams()
    assert lib.aeros_params_default(ctypes.byref(p)) == 0
    q = held_suarez_params()
    for name, _ in AerosParams._fields_:
        assert getattr(p, name) == getattr(q, name), name


def test_bad_arguments_return_codes(lib):
    """Argument errors come back as status codes, before any device work."""
    from aeros_gb300.params import held_suarez_params
    h = ctypes.c_void_p()
    assert lib.aeros_sht_create(ctypes.byref(h), 0, -1, -1, 1) == -1
    assert lib.aeros_sht_create(ctypes.byref(h), 21, -1, -1, 0) == -1
    for bad in (dict(dt=0.0), dict(ndiff=5), dict(tau_diff=0.0), dict(eps_filter=1.0), dict(raw_alpha=0.0),
                dict(si_alpha=0.4), dict(nmember=0)):
        p = held_suarez_params(trunc=21, nlev=12, **bad)
        assert lib.aeros_dyn_create(ctypes.byref(h), ctypes.byref(p), None, None) == -1, bad
    p = held_suarez_params(trunc=21, nlev=65)   # 2 to 64 levels
    assert lib.aeros_dyn_create(ctypes.byref(h), ctypes.byref(p), None, None) == -7
    # groups: no handles, or a null group
    g = ctypes.c_void_p()
    assert lib.aeros_group_create(ctypes.byref(g), None, 0) == -1
    assert lib.aeros_group_info(None, None, None, None) == -1
