"""Ensemble groups: members of different truncations stepped by one CUDA graph
per step (fused ragged launches, or one branch per handle) give bit-identical
states to stepping each handle on its own."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _make(trunc, nlev, members, seed0, precision=0):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn
    from tests.test_gpu_dyn import moving_state
    p = held_suarez_params(trunc=trunc, nlev=nlev, nmember=members, precision=precision)
    d = AerosDyn(p)
    o = OracleDyn(held_suarez_params(trunc=trunc, nlev=nlev))
    sts = [moving_state(o, seed=seed0 + e) for e in range(members)]
    st = [np.stack([s[i] for s in sts]) for i in range(4)]
    for e in range(members):
        d.set_member_forcing(e, 40.0 + 10 * e, 1.0 / (40 * 86400.0))
    d.set_state(*st)
    return d, st


@pytest.mark.parametrize("fuse", ["1", "0"])
@pytest.mark.parametrize("precision", [0, 1])
def test_group_matches_individual_handles(gpulib, precision, fuse, monkeypatch):
    from aeros_gb300.dynamics import AerosGroup
    monkeypatch.setenv("AEROS_GROUP_FUSE", fuse)
    cfg = [(21, 16, 2, 100), (31, 20, 2, 200), (42, 20, 2, 300)]
    grouped = [_make(*c, precision=precision)[0] for c in cfg]
    single = [_make(*c, precision=precision)[0] for c in cfg]
    g = AerosGroup(grouped)
    info = g.info()
    assert info["fused"] == (fuse == "1")
    g.step(4)
    for d in single:
        d.step(4)
    for a, b in zip(grouped, single):
        for x, y in zip(a.get_state(squeeze=False), b.get_state(squeeze=False)):
            assert np.array_equal(x, y)
        assert a.counters()[0] == b.counters()[0] == 4
    n = g.launch_count()
    assert n == info["kernels_startup"] + 3 * info["kernels_step"]
    if fuse == "1":
        # one ragged launch per kernel of the step over the three truncations
        assert info["kernels_step"] <= 8, info


@pytest.mark.parametrize("precision,members", [(0, 12), (1, 32)])
def test_fused_group_of_large_ensembles(gpulib, precision, members):
    """The batching configuration (32 members per truncation in the split form,
    where every handle takes the double-float column kernel; 12 in FP64), with
    the handles' launch shapes set apart: the fused group unifies them, steps
    with at most 8 launches (the spectral kernels of 16 and 20 levels stay
    apart) and stays bit-identical to the handles stepped alone."""
    from aeros_gb300.dynamics import AerosGroup
    cfg = [(21, 16, members, 700), (31, 20, members, 800), (42, 20, members, 900)]
    grouped = [_make(*c, precision=precision)[0] for c in cfg]
    single = [_make(*c, precision=precision)[0] for c in cfg]
    shapes = [dict(col_thr=128, spec_warps=2), dict(col_thr=64, spec_warps=8), dict(col_thr=256, spec_warps=4)]
    for a, b, sh in zip(grouped, single, shapes):
        a.set_tune_shapes(**sh)
        b.set_tune_shapes(**sh)
    g = AerosGroup(grouped)
    info = g.info()
    assert info["fused"] and info["kernels_step"] <= 8, info
    g.step(3)
    for d in single:
        d.step(3)
    for a, b in zip(grouped, single):
        for x, y in zip(a.get_state(squeeze=False), b.get_state(squeeze=False)):
            assert np.array_equal(x, y)


def test_smaller_handle_created_later_keeps_larger_launches(gpulib):
    """A kernel's shared-memory limit is per function: creating a smaller split
    handle after a larger one must not shrink what the larger one launches with."""
    big, _ = _make(42, 20, 1, 500, precision=1)
    ref, _ = _make(42, 20, 1, 500, precision=1)
    ref.step(2)
    small, _ = _make(21, 16, 1, 600, precision=1)
    small.step(1)
    big.step(2)
    for x, y in zip(big.get_state(), ref.get_state()):
        assert np.array_equal(x, y)


def test_fused_group_of_more_handles_than_one_launch_takes(gpulib):
    """Six handles (one launch fuses at most four): the launches split into
    parts of four and two, and the states stay bit-identical."""
    from aeros_gb300.dynamics import AerosGroup
    cfg = [(21, 16, 1, 1000 + i) for i in range(4)] + [(31, 20, 1, 1100), (42, 20, 1, 1200)]
    grouped = [_make(*c)[0] for c in cfg]
    single = [_make(*c)[0] for c in cfg]
    g = AerosGroup(grouped)
    info = g.info()
    assert info["fused"] and 7 < info["kernels_step"] <= 21, info
    g.step(3)
    for d in single:
        d.step(3)
    for a, b in zip(grouped, single):
        for x, y in zip(a.get_state(squeeze=False), b.get_state(squeeze=False)):
            assert np.array_equal(x, y)


def test_group_with_a_many_level_handle(gpulib):
    """A handle of 40 levels beside one of 16 in a fused group: its column and
    spectral kernels differ from the others', so they launch apart, and every
    state equals stepping the handles on their own."""
    from aeros_gb300.dynamics import AerosGroup
    cfg = [(21, 16, 2, 400), (21, 40, 2, 500)]
    grouped = [_make(*c)[0] for c in cfg]
    single = [_make(*c)[0] for c in cfg]
    g = AerosGroup(grouped)
    g.step(3)
    for d in single:
        d.step(3)
    for a, b in zip(grouped, single):
        for x, y in zip(a.get_state(squeeze=False), b.get_state(squeeze=False)):
            assert np.array_equal(x, y)
