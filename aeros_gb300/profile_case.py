"""A fixed step workload for profiling one kernel under ncu.

  python -m aeros_gb300.profile_case --trunc 42 --nlev 20 --members 16 --steps 3 [--precision fp64|split]
                                    [--shapes spec_cols=1,spec_warps=2]

Builds an ensemble of Held-Suarez members (rest + 0.1 K noise, one seed per
member) and runs `steps` steps with direct launches (no graph), so that an
ncu `-k <kernel> -s <n> -c <k>` selection sees a small, fixed number of
launches.  With 16 members at T42L20 the grid fields of one launch (~235 MB)
exceed the 129 MB L2, so DRAM counters measure real traffic.
"""
import argparse
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--trunc", type=int, default=42)
    ap.add_argument("--nlev", type=int, default=20)
    ap.add_argument("--members", type=int, default=16)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--transport", action="store_true",
                    help="run `steps` tracer-transport calls (one member's grid) instead of dynamics steps")
    ap.add_argument("--tune", action="store_true", help="run the launch-shape autotuner before stepping")
    ap.add_argument("--shapes", default="",
                    help="launch shapes to set before stepping, e.g. spec_cols=1,spec_warps=2 (AerosDyn.TUNE_KEYS)")
    ap.add_argument("--sht-batch", type=int, default=0,
                    help="run `steps` scalar synthesis + analysis pairs of this many fields at --trunc instead")
    ap.add_argument("--adjoint", action="store_true",
                    help="run one checkpointed forward/backward window of `steps` steps (checkpoints every "
                         "--every) of one member instead")
    ap.add_argument("--every", type=int, default=4)
    ap.add_argument("--packed", action="store_true",
                    help="take the steps through aeros_dyn_step_packed between page-locked host arrays "
                         "(the end-to-end form: copy-in kernel, step, copy-out kernel in one graph)")
    a = ap.parse_args(argv)
    if a.transport:
        return transport_case(a)
    if a.adjoint:
        return adjoint_case(a)
    if a.sht_batch > 0:
        return sht_case(a)
    from .params import held_suarez_params, PREC_FP64, PREC_SPLIT
    from .dynamics import AerosDyn
    from .spectral import AerosSHT
    p = held_suarez_params(trunc=a.trunc, nlev=a.nlev, nmember=a.members,
                           precision=PREC_SPLIT if a.precision == "split" else PREC_FP64)
    dyn = AerosDyn(p)
    if a.shapes:
        dyn.set_tune_shapes(**{k: int(v) for k, v in (kv.split("=") for kv in a.shapes.split(","))})
    sht = AerosSHT(a.trunc, batch_max=a.nlev)
    dyn.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = dyn.get_state(squeeze=False)
    t = t.copy()
    for e in range(a.members):
        rng = np.random.default_rng(e)
        tg = sht.synthesis(t[e]) + rng.normal(0.0, 0.1, (a.nlev, dyn.nlat, dyn.nlon))
        t[e] = sht.analysis(tg)
    dyn.set_state(vor, div, t, lnps)
    if a.tune:
        before, after, shapes = dyn.autotune(reps=3)
        print(f"autotune: {before:.4f} -> {after:.4f} ms/step with {shapes}")
    if a.packed:
        return packed_case(a, dyn)
    for _ in range(a.steps):
        ks = dyn.profile_step()
    print(" ".join(f"{n}={ms:.4f}ms" for n, ms in ks))
    return 0


def packed_case(a, dyn):
    """`steps` steps through aeros_dyn_step_packed with page-locked host arrays
    (the one-graph form), after two direct steps."""
    import ctypes
    import time
    dyn.step(2)
    n = dyn.state_size()
    arrs = []
    for src in (dyn.pack(*dyn.get_state(squeeze=False)), dyn.pack(*dyn.get_old_state(squeeze=False)), None, None):
        x = np.empty(n, np.complex128) if src is None else src.copy()
        dyn.host_register(x)
        arrs.append(x)
    now, old, now_out, old_out = arrs
    nstep = dyn.counters()[0]
    t0 = time.perf_counter()
    for _ in range(a.steps):
        dyn.step_packed(now, old, nstep, 1, now_out, old_out)
        now, now_out = now_out, now
        old, old_out = old_out, old
        nstep += 1
    t1 = time.perf_counter()
    print(f"packed steps: {a.steps}, {1e3 * (t1 - t0) / a.steps:.4f} ms per step (host clock)")
    for x in arrs:
        dyn.host_unregister(x)
    return 0


def adjoint_case(a):
    """The differentiation form's window pair on one member: a seeded
    red-spectrum state (vorticity 1e-5/l^2, divergence 0.2 of it, temperature
    1 K/l about 264 K, seed 2), window_forward(steps, every), window_backward;
    the wall times are printed."""
    import time
    from .params import held_suarez_params
    from .dynamics import AerosDyn
    from .spectral import AerosSHT
    d = AerosDyn(held_suarez_params(trunc=a.trunc, nlev=a.nlev))
    s = AerosSHT(a.trunc, batch_max=1)
    rng = np.random.default_rng(2)
    L, M = np.asarray(s.l_of_lm, float), np.asarray(s.m_of_lm)

    def red(shape, slope):
        c = (rng.standard_normal(shape + (len(L),)) + 1j * rng.standard_normal(shape + (len(L),))) * (L + 1) ** slope
        c[..., M == 0] = c[..., M == 0].real
        return c
    d.set_isothermal(264.0, 1.0e5)
    _, _, t, lnps = d.get_state()
    vor, div = 1e-5 * red((d.nlev,), -2.0), 2e-6 * red((d.nlev,), -2.0)
    vor[:, 0] = 0
    div[:, 0] = 0
    d.set_state(vor, div, t + red((d.nlev,), -1.0), lnps)
    t0 = time.perf_counter()
    J = d.window_forward(a.steps, a.every)
    t1 = time.perf_counter()
    d.window_backward()
    t2 = time.perf_counter()
    print(f"adjoint window: {a.steps} steps, J {float(J[0]):.6e}, forward {1e3 * (t1 - t0):.2f} ms, "
          f"backward {1e3 * (t2 - t1):.2f} ms")
    return 0


def sht_case(a):
    """Scalar transforms of seeded red-spectrum fields (Var ~ (l+1)^-3, seed 1) on
    device arrays, in the chosen precision: `steps` synthesis + analysis pairs."""
    import torch
    from .spectral import AerosSHT
    from .params import PREC_SPLIT, PREC_FP64
    s = AerosSHT(a.trunc, batch_max=a.sht_batch)
    s.set_precision(PREC_SPLIT if a.precision == "split" else PREC_FP64)
    L = np.asarray(s.l_of_lm, float)
    M = np.asarray(s.m_of_lm)
    rng = np.random.default_rng(1)
    c = (rng.standard_normal((a.sht_batch, s.nlm)) + 1j * rng.standard_normal((a.sht_batch, s.nlm))) * (L + 1) ** -1.5
    c[:, M == 0] = c[:, M == 0].real
    cd = torch.from_numpy(c).cuda()
    for _ in range(a.steps):
        g = s.synthesis(cd)
        s.analysis(g)
    torch.cuda.synchronize()
    print(f"sht T{a.trunc} batch={a.sht_batch} pairs={a.steps} precision={a.precision}")
    return 0


def transport_case(a):
    """The bench's transport workload: winds of a 35 m/s solid-body rotation
    plus a divergent part and 2 m/s seeded noise, the wavenumber-1 surface
    pressure of the reference's transport test, the blob tracer of the bench
    (0.002 + 0.015 exp(-6 r^2)), dt = 1800 s, device arrays; `steps` calls of
    AerosTransport.step."""
    import torch
    from .params import held_suarez_params
    from .dynamics import AerosDyn
    from .transport import AerosTransport
    d = AerosDyn(held_suarez_params(trunc=a.trunc, nlev=a.nlev))
    nlev, nlat, nlon = d.nlev, d.nlat, d.nlon
    lon = 2.0 * np.pi * np.arange(nlon) / nlon
    lat = np.arcsin(d.sinlat)
    rng = np.random.default_rng(7)
    k = (np.arange(1, nlev + 1) / nlev)[:, None, None]
    u = (35.0 * np.cos(lat)[None, :, None] + 35.0 * np.sin(lon)[None, None, :] * np.cos(lat)[None, :, None] * k
         + rng.normal(0.0, 2.0, (nlev, nlat, nlon)))
    v = 17.5 * np.cos(lon)[None, None, :] + rng.normal(0.0, 2.0, (nlev, nlat, nlon))
    lnps = np.log(1.0e5 * (1.0 + 0.05 * np.sin(lon)[None, :] * np.cos(lat)[:, None]))
    r2 = (lon[None, :] - np.pi) ** 2 + 4.0 * lat[:, None] ** 2
    q = np.broadcast_to(0.002 + 0.015 * np.exp(-6.0 * r2), (nlev, nlat, nlon)).copy()
    g = AerosTransport(a.trunc, d.A, d.B)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (u, v, lnps, q)]
    for _ in range(a.steps):
        g.step(*dev, 1800.0)
    torch.cuda.synchronize()
    cfl, nsub = g.last()
    print(f"transport calls={a.steps} max_courant={cfl:.3f} substeps={nsub}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
