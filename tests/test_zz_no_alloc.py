"""The allocation-free synthesis entry point against the regular one.

aeros_sht_synthesis_noalloc exists for callers that cannot call cudaMalloc
(device memory owned by another allocator or reserved up front, or a loop whose
memory must stay fixed): its scratch lives in static device arrays.  It must
give the same fields as aeros_sht_synthesis (FP64 bar, 1e-12 relative) on two
calls in a row, since every call reuses the same static arrays, and it must
refuse sizes beyond its fixed scratch.  This file sorts last so that a run
stopping at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from tests._helpers import red_spectrum

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_synthesis_matches_regular(gpulib):
    torch = pytest.importorskip("torch")
    from aeros_gb300 import _capi
    from aeros_gb300.spectral import AerosSHT
    L = _capi.lib()
    sht = AerosSHT(42, batch_max=12)
    rng = np.random.default_rng(2024)
    nb = 12
    for _ in range(2):
        c = torch.from_numpy(red_spectrum(rng, sht.l_of_lm, sht.m_of_lm, (nb,))).cuda()
        ref = sht.synthesis(c)
        out = torch.full((nb, sht.nlat, sht.nlon), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.aeros_sht_synthesis_noalloc(sht._h, _p(c), _p(out), nb)
        assert rc == _capi.OK, _capi.lib().aeros_last_error()
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(a).all()
        assert np.max(np.abs(a - b)) / np.max(np.abs(b)) <= 1e-12


def test_noalloc_rejects_out_of_range(gpulib):
    torch = pytest.importorskip("torch")
    from aeros_gb300 import _capi
    from aeros_gb300.spectral import AerosSHT
    L = _capi.lib()
    sht = AerosSHT(42, batch_max=1)
    c = torch.zeros((1, sht.nlm), dtype=torch.complex128, device="cuda")
    f = torch.zeros((1, sht.nlat, sht.nlon), dtype=torch.float64, device="cuda")
    assert L.aeros_sht_synthesis_noalloc(sht._h, _p(c), _p(f), 257) == _capi.ERR_ARG
    assert L.aeros_sht_synthesis_noalloc(sht._h, _p(c), _p(f), 0) == _capi.ERR_ARG
    host = np.zeros((1, sht.nlm), np.complex128)
    assert L.aeros_sht_synthesis_noalloc(sht._h, host.ctypes.data_as(ctypes.c_void_p), _p(f), 1) == _capi.ERR_ARG
    big = AerosSHT(341, batch_max=1)        # nlat 512 x 342: 2^19 entries hold 2 fields, not 3
    c3 = torch.zeros((3, big.nlm), dtype=torch.complex128, device="cuda")
    f3 = torch.zeros((3, big.nlat, big.nlon), dtype=torch.float64, device="cuda")
    assert L.aeros_sht_synthesis_noalloc(big._h, _p(c3), _p(f3), 3) == _capi.ERR_ARG
