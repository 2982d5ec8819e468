#!/usr/bin/env python
"""Benchmark: simulated years per day (SYPD) of the dry Held-Suarez spectral
step at T42L20 (128x64 Gaussian grid, 20 sigma levels, dt = 1800 s), one step
= one pass of the transform-method step over one model state.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

GPU arm: the C-ABI library (include/aeros_gpu.h) steps the state held in HBM;
each timed step is preceded by an L2 flush (a 256 MB write) outside its CUDA
event pair.  `e2e` is the same metric through the C-ABI with pinned HOST
buffers: per step the two time levels go host->device, one step runs, and the
new state comes back device->host.  Reference arm: the CPU restatement of the
reference's OpenMP path (oracle/), all host threads.  With N > 1 (torchrun)
every rank steps its own replica; value is the sum over ranks and time the
max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

STEPS_PER_YEAR = 365.25 * 86400.0 / 1800.0      # src/aeros_defs.f90:100, dt = 1800 s
METRIC = "simulated years/day at T42L20, FP64 vs split-prec/batched, at <=1e-10 rel err"


def sypd(t_step_s):
    return 86400.0 / (STEPS_PER_YEAR * t_step_s)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--trunc", type=int, default=42)
    ap.add_argument("--nlev", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=60)
    ap.add_argument("--no-split", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-steps", type=int, default=20)
    ap.add_argument("--t42-handles", type=int, default=3, choices=[1, 2, 3, 4, 6, 8, 12],
                    help="handles the 96 T42L20 members are split into")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the T85/T170/T341 transform sweep")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner of the batched form")
    ap.add_argument("--shapes-from-cache", action="store_true",
                    help="take every handle's launch shapes from the AEROS_TUNE_CACHE file written by an earlier "
                         "run (handles load them when created) instead of timing candidates; for profiling the "
                         "same shapes under ncu")
    ap.add_argument("--no-transport", action="store_true", help="skip the tracer-transport measurement")
    a = ap.parse_args()
    if a.shapes_from_cache:
        if not os.environ.get("AEROS_TUNE_CACHE"):
            ap.error("--shapes-from-cache needs AEROS_TUNE_CACHE")
        a.no_tune = True
    return a


def reduce_time(local_s, world, backend="nccl"):
    """Max over ranks of a per-rank time (the replicas share no data)."""
    if world <= 1:
        return local_s
    import torch
    import torch.distributed as dist
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([float(local_s)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- peaks
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def fp64_peak_tflops(torch):
    """Live FP64 throughput of this GPU: cuBLAS DGEMM 4096^3 (best of 5)."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * 4096 ** 3 / best / 1e12


# ---------------------------------------------------------------- work model
# FP64 flops of the column terms and Held-Suarez forcing per grid point and
# level: ncu's count for the one-lane column kernel at T42L20 x 16 members
# (dadd + dmul + 2 dfma thread instructions, 260.4 M per launch), divided by
# the points and levels.  It includes the operations of the exp and log calls.
COLUMN_FP64_FLOPS_PER_POINT_LEVEL = 99.35

# FP64-pipe issue slots (warp instructions on the FP64 pipe x 32) per grid cell
# of the tracer transport at T42L20 on the bench's workload, from ncu's
# sm__inst_executed_pipe_fp64 count: per call (k_tr_begin 9.8, k_tr_courant
# 25.8, k_tr_winds 8.9) and per sub-step (k_tr_zonal 25.0, k_tr_mfaces 13.7,
# k_tr_vert 29.3).  Every FP64 warp instruction holds the pipe for 16 cycles (2
# lanes per clock per SM), whether it is an add, a multiply, an FMA or a compare.
TRANSPORT_FP64_SLOTS_PER_CELL = {"call": 44.5, "substep": 68.0}
FP64_LANES_PER_CLOCK_PER_SM = 2


def kernel_work(T, nlat, nlon, nlm, nlev):
    """Algorithmic work per launch of each step kernel at one member:
    flops for the contractions, FFTs and column terms (FP64, the pipe that
    bounds them on GB300), bytes for the memory-bound ones.
    F_leg = 2 nlat nlm flops per scalar Legendre sum (hemisphere-folded);
    FFT = 2.5 nlon log2(nlon) flops per real row."""
    import math
    F_leg = 2.0 * nlat * nlm
    fft = 2.5 * nlon * math.log2(nlon)
    ng = nlon * nlat
    st_bytes = (3 * nlev * nlm + nlm) * 16
    return {
        "legendre_synth": ("flops", F_leg * (8 * nlev + 2)),
        "fourier_synth": ("flops", fft * nlat * (7 * nlev + 3)),
        "column": ("flops", COLUMN_FP64_FLOPS_PER_POINT_LEVEL * ng * nlev),
        "fourier_anal": ("flops", fft * nlat * (4 * nlev + 1)),
        "legendre_anal": ("flops", F_leg * (6 * nlev + 1)),
        "spectral": ("bytes", 5.0 * st_bytes),
        "mass": ("flops", F_leg + 2 * fft * 1.0),
    }


def initial_state(dyn, sht, seed):
    """Held-Suarez start: rest, T = 264 K, ps = 1000 hPa, N(0, 0.1^2) K on grid T."""
    import numpy as np
    dyn.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = dyn.get_state()
    rng = np.random.default_rng(seed)
    tg = sht.synthesis(t) + rng.normal(0.0, 0.1, (dyn.nlev, dyn.nlat, dyn.nlon))
    return vor, div, sht.analysis(tg), lnps


def time_steps(stepper, stream, K, torch, flush=None):
    """Mean device time per step over K steps (CUDA events on `stream`); with
    `flush`, a >L2 write precedes every step outside its event pair."""
    if flush is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            stepper.step_async(K)
            e1.record(stream)
        stepper.sync()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / K
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    with torch.cuda.stream(stream):
        for i in range(K):
            flush.fill_(i & 0xFF)
            ev0[i].record(stream)
            stepper.step_async(1)
            ev1[i].record(stream)
    stepper.sync()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)) / 1e3 / K


def split_form(args, sht, dyn_fp64, flush, torch):
    """T42L20 single member with the split-precision Legendre contractions:
    SYPD with the same flushed timing, and the relative difference from the
    FP64 GPU path after the same steps from the same state."""
    import numpy as np
    from aeros_gb300.params import held_suarez_params, PREC_SPLIT
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=args.trunc, nlev=args.nlev, precision=PREC_SPLIT)
    d = AerosDyn(p)
    ref = AerosDyn(held_suarez_params(trunc=args.trunc, nlev=args.nlev))
    st = initial_state(d, sht, seed=0)
    d.set_state(*st)
    ref.set_state(*st)
    d.step(24)
    ref.step(24)
    err = max(float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(d.get_state(), ref.get_state()))
    s = torch.cuda.Stream()
    d.set_stream(s.cuda_stream)
    if not args.no_tune:
        d.autotune(reps=5)
    d.step_async(3)
    d.sync()
    t = time_steps(d, s, args.steps, torch, flush)
    return {"sypd": sypd(t), "ms_per_step": t * 1e3,
            "max_rel_diff_vs_fp64_gpu_after_24_steps": err,
            "legendre": "tcgen05 bf16 Ozaki digits (55 bits), exact int64 recombination"}


def transform_sweep(args, torch):
    """Standalone transforms at T85, T170 and T341 (256x128, 512x256, 1024x512
    grids), batch 240 = 30 levels x 8 fields of seeded complex Gaussian
    coefficients with variance proportional to (l+1)^-3 and real m = 0 (seed 1),
    device pointers.  FP64 and split precision: synthesis and analysis time
    (CUDA events on the handle's stream, mean of 5 after 2 warm-up calls), the
    FP64-equivalent Legendre rate 2 nlat nlm B / t per direction, the split
    form's relative difference from the FP64 path and its round-trip error."""
    import numpy as np
    from aeros_gb300 import _capi
    from aeros_gb300.spectral import AerosSHT, _ptr
    L = _capi.lib()
    B = 240
    out = {"batch": B}
    stream = torch.cuda.Stream()
    for T in (85, 170, 341):
        hs = [AerosSHT(T, batch_max=B, precision=p) for p in (0, 1)]
        for h in hs:
            _capi.check(L.aeros_sht_set_stream(h._h, ctypes_void(stream.cuda_stream)), "aeros_sht_set_stream")
        h0 = hs[0]
        rng = np.random.default_rng(1)
        l = np.asarray(h0.l_of_lm, float)
        c = (rng.standard_normal((B, h0.nlm)) + 1j * rng.standard_normal((B, h0.nlm))) * (l + 1.0) ** -1.5
        c[:, np.asarray(h0.m_of_lm) == 0] = c[:, np.asarray(h0.m_of_lm) == 0].real
        cd = torch.from_numpy(c).cuda()
        g = [torch.empty((B, h0.nlat, h0.nlon), dtype=torch.float64, device="cuda") for _ in hs]
        cb = [torch.empty_like(cd) for _ in hs]
        torch.cuda.synchronize()

        def timeit(fn):
            for _ in range(2):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(5):
                fn()
            e1.record(stream)
            e1.synchronize()
            return e0.elapsed_time(e1) / 5.0
        res = {}
        flops = 2.0 * h0.nlat * h0.nlm * B
        for i, name in enumerate(("fp64", "split")):
            h = hs[i]
            ts = timeit(lambda: _capi.check(L.aeros_sht_synthesis(h._h, _ptr(cd), _ptr(g[i]), B), "synthesis"))
            ta = timeit(lambda: _capi.check(L.aeros_sht_analysis(h._h, _ptr(g[i]), _ptr(cb[i]), B), "analysis"))
            res[name] = {"synthesis_ms": ts, "analysis_ms": ta,
                         "legendre_equiv_gflops_synthesis": flops / (ts * 1e-3) / 1e9,
                         "legendre_equiv_gflops_analysis": flops / (ta * 1e-3) / 1e9}
        torch.cuda.synchronize()
        rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
        # split analysis of the split synthesis -> round trip; FP64 path as the reference point
        res["split_vs_fp64_synthesis"] = rel(g[1], g[0])
        res["split_vs_fp64_analysis"] = rel(cb[1], cb[0])
        res["split_round_trip"] = rel(cb[1], cd)
        res["fp64_round_trip"] = rel(cb[0], cd)
        res["grid"] = f"{h0.nlon}x{h0.nlat}"
        # the CPU oracle's timing build on the host cores, 16 of the 240 fields (one per thread), scaled to 240
        res["cpu_oracle"] = oracle_sweep_time(T, c[:16], B)
        out[f"T{T}"] = res
        del hs, g, cb, cd
    return out


def oracle_sweep_time(T, c16, B):
    """Synthesis and analysis time of the CPU oracle's timing build (OpenMP over
    fields, all host cores) for a sample of fields, scaled to a batch of B."""
    import numpy as np
    import oracle.pyoracle as po
    cores, _ = host_cpu()
    po.use_variant("fast")
    po.set_threads(cores)
    s = po.OracleSHT(T)
    n = len(c16)
    f = s.synthesis(c16)
    s.analysis(f)
    t0 = time.perf_counter()
    f = s.synthesis(c16)
    ts = time.perf_counter() - t0
    t0 = time.perf_counter()
    s.analysis(f)
    ta = time.perf_counter() - t0
    return {"synthesis_ms": ts * 1e3 * B / n, "analysis_ms": ta * 1e3 * B / n, "cores": cores, "kind": "port",
            "sample": f"{n} fields on {cores} threads (one field per thread), scaled to {B}"}


def ctypes_void(p):
    import ctypes
    return ctypes.c_void_p(p)


def adjoint_form(args):
    """Differentiation form: gradient of the window-mean kinetic energy over a
    96-step T42L20 window (dt 1800 s, checkpoints every 12 steps) from a seeded
    red-spectrum state (vorticity 1e-5/l^2 s^-1, divergence 0.2 of it,
    temperature 1 K/l about 264 K, seed 2); forward and backward wall time
    (synchronised) and a central-difference check of dJ/dk_a."""
    import numpy as np
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300.spectral import AerosSHT
    d = AerosDyn(held_suarez_params(trunc=args.trunc, nlev=args.nlev))
    s = AerosSHT(args.trunc, batch_max=1)
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
    x0 = (vor, div, t + red((d.nlev,), -1.0), lnps)
    nst, every = 96, 12
    ka0 = d.params.hs_k_a

    def J(ka=ka0):
        d.set_member_forcing(0, d.params.hs_dt_y, ka)
        d.set_mass_target(-1.0)
        d.set_state(*x0)
        return float(d.window_forward(nst, every)[0])
    J()
    d.window_backward()   # warm-up
    t0 = time.perf_counter()
    j0 = J()
    t1 = time.perf_counter()
    _, _, ka_b, dty_b = d.window_backward()
    t2 = time.perf_counter()
    e = 1e-4 * ka0
    fd = (J(ka0 + e) - J(ka0 - e)) / (2 * e)
    return {"workload": f"T{args.trunc}L{args.nlev} window of {nst} steps, checkpoints every {every}",
            "J": j0, "forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
            "backward_over_forward": (t2 - t1) / (t1 - t0), "dJ_dka": float(ka_b[0]), "dJ_ddTy": float(dty_b[0]),
            "fd_rel_err_ka": abs(fd - ka_b[0]) / abs(ka_b[0]),
            # the oracle has no adjoint: the CPU reference point is the forward window's steps on all host cores
            "cpu_oracle_forward_ms": oracle_step_time(args, host_cpu()[0], nst) * nst * 1e3}


def transport_form(args, torch):
    """Tracer transport (the grid tracer of the moist model) at T42L20, dt 1800 s:
    winds of a 35 m/s solid-body rotation plus a divergent part and 2 m/s seeded
    noise, the wavenumber-1 surface pressure and a blob tracer of the
    reference's transport test; device-resident arrays, one synchronised call
    per sample (the call reads the Courant number back to size its sub-steps).
    The numpy oracle's time for the same call is the CPU line beside it."""
    import numpy as np
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.transport import AerosTransport
    d = AerosDyn(held_suarez_params(trunc=args.trunc, nlev=args.nlev))
    s = AerosSHT(args.trunc, batch_max=1)
    nlev, nlat, nlon = d.nlev, d.nlat, d.nlon
    lon = 2.0 * np.pi * np.arange(nlon) / nlon
    lat = np.arcsin(np.asarray(s.sinlat))
    rng = np.random.default_rng(7)
    k = (np.arange(1, nlev + 1) / nlev)[:, None, None]
    u = (35.0 * np.cos(lat)[None, :, None] + 35.0 * np.sin(lon)[None, None, :] * np.cos(lat)[None, :, None] * k
         + rng.normal(0.0, 2.0, (nlev, nlat, nlon)))
    v = 17.5 * np.cos(lon)[None, None, :] + rng.normal(0.0, 2.0, (nlev, nlat, nlon))
    lnps = np.log(1.0e5 * (1.0 + 0.05 * np.sin(lon)[None, :] * np.cos(lat)[:, None]))
    r2 = (lon[None, :] - np.pi) ** 2 + 4.0 * lat[:, None] ** 2
    q = np.broadcast_to(0.002 + 0.015 * np.exp(-6.0 * r2), (nlev, nlat, nlon)).copy()
    A, B = d.A, d.B
    g = AerosTransport(args.trunc, A, B)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (u, v, lnps, q)]
    for _ in range(3):
        g.step(*dev, 1800.0)
    torch.cuda.synchronize()
    n = 20
    t0 = time.perf_counter()
    for _ in range(n):
        g.step(*dev, 1800.0)
    torch.cuda.synchronize()
    t_gpu = (time.perf_counter() - t0) / n
    cfl, nsub = g.last()
    from oracle.transport_oracle import OracleTransport
    o = OracleTransport(np.asarray(s.sinlat), np.asarray(s.gauss_w), nlon, A, B)
    o.transport(u, v, lnps, q, 1800.0)
    t0 = time.perf_counter()
    for _ in range(3):
        o.transport(u, v, lnps, q, 1800.0)
    t_cpu = (time.perf_counter() - t0) / 3
    cells = nlev * nlat * nlon
    # algorithmic bytes of one sub-step: zonal 6, meridional 5, vertical 6 doubles per cell
    sub_bytes = 17 * 8 * cells
    # the bound: FP64-pipe issue slots (ncu's count per cell) at 2 lanes per clock per SM
    props = torch.cuda.get_device_properties(0)
    sm_hz = getattr(props, "clock_rate", 0) * 1e3 or 2.07e9
    slots = cells * (TRANSPORT_FP64_SLOTS_PER_CELL["call"] + TRANSPORT_FP64_SLOTS_PER_CELL["substep"] * nsub)
    pipe_s = slots / (FP64_LANES_PER_CLOCK_PER_SM * props.multi_processor_count * sm_hz)
    return {"workload": f"T{args.trunc}L{nlev} grid {nlon}x{nlat}, dt 1800 s, device arrays", "ms_per_call": t_gpu * 1e3,
            "max_courant": cfl, "substeps": nsub, "cell_substeps_per_s": cells * nsub / t_gpu,
            "achieved_GBs": sub_bytes * nsub / t_gpu / 1e9, "bytes_per_substep": sub_bytes,
            "roofline": {"bound": "fp64 pipe issue", "fp64_pipe_ms": pipe_s * 1e3, "frac": pipe_s / t_gpu,
                         "sm_clock_ghz": sm_hz / 1e9,
                         "note": "FP64-pipe slots per cell from ncu; the call also holds one host read of the "
                                 "Courant number"},
            "cpu_oracle_ms_per_call": t_cpu * 1e3, "cpu_oracle": "numpy restatement, 1 core"}


def build_members(cfg, prec, seed_base, tune, autotune_log):
    """Ensemble handles: one per (T, L, n) of cfg, n members each, every member
    with its own seed (rest, 264 K, 1000 hPa, N(0, 0.1^2) K grid noise) and
    equator-pole contrast dT_y ~ U(40, 80) K; launch shapes autotuned outside
    any timed region."""
    import numpy as np
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300.spectral import AerosSHT
    rng = np.random.default_rng(seed_base)
    hs, seed = [], seed_base
    for T, L, n in cfg:
        d = AerosDyn(held_suarez_params(trunc=T, nlev=L, nmember=n, precision=prec))
        sht = AerosSHT(T, batch_max=L)
        d.set_isothermal(264.0, 1.0e5)
        vor, div, t, lnps = d.get_state(squeeze=False)
        t = t.copy()
        for e in range(n):
            r = np.random.default_rng(seed)
            seed += 1
            t[e] = sht.analysis(sht.synthesis(t[e]) + r.normal(0.0, 0.1, (L, d.nlat, d.nlon)))
            d.set_member_forcing(e, rng.uniform(40.0, 80.0), 1.0 / (40.0 * 86400.0))
        d.set_state(vor, div, t, lnps)
        if tune:
            b0, b1, shp = d.autotune(reps=3)
            autotune_log[f"T{T}L{L}x{n}"] = {"ms_before": b0, "ms_after": b1, "shapes": shp}
        hs.append(d)
    return hs


def time_group(hs, steps, torch, fuse=True):
    """Device time per step of a group of handles: fused launches (one per kernel
    over the handles) or, with fuse=False, one graph branch per handle."""
    from aeros_gb300.dynamics import AerosGroup
    prev = os.environ.get("AEROS_GROUP_FUSE")
    os.environ["AEROS_GROUP_FUSE"] = "1" if fuse else "0"
    try:
        g = AerosGroup(hs)
    finally:
        if prev is None:
            del os.environ["AEROS_GROUP_FUSE"]
        else:
            os.environ["AEROS_GROUP_FUSE"] = prev
    s = torch.cuda.Stream()
    g.set_stream(s.cuda_stream)
    g.step_async(3)
    g.sync()
    n0 = g.launch_count()
    t = time_steps(g, s, steps, torch)
    launches = (g.launch_count() - n0) / steps
    time_group.last_info = g.info()
    del g
    return t, launches


def batched_form(args, torch, t_single):
    """The batching form.  (1) T42L20 ensembles: 96 members of the headline
    configuration (each its own seed and dT_y), one CUDA graph launch per step,
    FP64 and split precision, as 3 handles of 32 (the group fuses their
    launches: one ragged launch per kernel over the handles; the split ones
    also as one graph branch per handle) and the split members also as one
    handle of 96 (one launch per kernel type and step); the best split
    aggregate SYPD over the single-member FP64
    path's is the ratio the >= 20x target is stated for.  (2) The mixed
    configuration of 96 uneven members, 32 x T21L16 + 32 x T31L20 + 32 x
    T42L20, FP64 and split, each with fused launches and as one graph branch
    per handle, beside the same members stepped one by one through
    the single-member FP64 path (32 x the step time of one member of each
    configuration).  Working sets > L2, so no flush is needed."""
    from aeros_gb300.params import held_suarez_params, PREC_FP64, PREC_SPLIT
    from aeros_gb300.dynamics import AerosDyn
    out = {"steps": args.batched_steps}
    tunelog = {}
    # (1) T42L20 ensembles
    nh = args.t42_handles
    per = 96 // nh
    t42 = {"members": f"96 x T42L20 ({nh} handles of {per})"}
    for name, prec in (("fp64", PREC_FP64), ("split", PREC_SPLIT)):
        hs = build_members([(42, 20, per)] * nh, prec, 5000, not args.no_tune, tunelog.setdefault("t42_" + name, {}))
        if prec == PREC_SPLIT and nh > 1:
            # the same handles as one graph branch each (before fusion unifies their launch shapes)
            tb, nlb = time_group(hs, args.batched_steps, torch, fuse=False)
            t42["split_branches"] = {"sypd": 96 * sypd(tb), "ms_per_step": tb * 1e3, "us_per_member_step": tb * 1e6 / 96,
                                     "gpu_launches_per_step": nlb, "fused_launches": False,
                                     "vs_fp64_single": 96 * sypd(tb) / sypd(t_single)}
        t, nl = time_group(hs, args.batched_steps, torch)
        del hs
        t42[name] = {"sypd": 96 * sypd(t), "ms_per_step": t * 1e3, "us_per_member_step": t * 1e6 / 96,
                     "gpu_launches_per_step": nl, "fused_launches": time_group.last_info["fused"],
                     "vs_fp64_single": 96 * sypd(t) / sypd(t_single)}
    # the same 96 split members as one handle: one launch per kernel type and step
    if nh != 1:
        hs = build_members([(42, 20, 96)], PREC_SPLIT, 5000, not args.no_tune, tunelog.setdefault("t42_split_1x96", {}))
        t, nl = time_group(hs, args.batched_steps, torch)
        del hs
        t42["split_one_handle"] = {"sypd": 96 * sypd(t), "ms_per_step": t * 1e3, "us_per_member_step": t * 1e6 / 96,
                                   "gpu_launches_per_step": nl, "vs_fp64_single": 96 * sypd(t) / sypd(t_single)}
    out["t42l20"] = t42
    out["vs_fp64_single_T42L20"] = max(v["vs_fp64_single"] for k, v in t42.items() if k.startswith("split"))
    # (2) the mixed configuration
    cfg = [(21, 16, 32), (31, 20, 32), (42, 20, 32)]
    mixed = {"members": "32 x T21L16 + 32 x T31L20 + 32 x T42L20"}
    for name, prec in (("fp64", PREC_FP64), ("split", PREC_SPLIT)):
        hs = build_members(cfg, prec, 1000, not args.no_tune, tunelog.setdefault("mixed_" + name, {}))
        tb, nlb = time_group(hs, args.batched_steps, torch, fuse=False)
        mixed[name + "_branches"] = {"sypd": 96 * sypd(tb), "ms_per_step": tb * 1e3, "gpu_launches_per_step": nlb,
                                     "fused_launches": False, "vs_fp64_single_mixed": 96 * sypd(tb) / sypd(t_single)}
        t, nl = time_group(hs, args.batched_steps, torch)
        del hs
        mixed[name] = {"sypd": 96 * sypd(t), "ms_per_step": t * 1e3, "gpu_launches_per_step": nl,
                       "fused_launches": time_group.last_info["fused"],
                       "vs_fp64_single_mixed": 96 * sypd(t) / sypd(t_single)}
    seq = 0.0
    perm = {}
    for T, L, n in cfg:
        d = AerosDyn(held_suarez_params(trunc=T, nlev=L))
        d.set_isothermal(264.0, 1.0e5)
        d.hs_perturb(1.0)
        if not args.no_tune:
            d.autotune(reps=3)
        s = torch.cuda.Stream()
        d.set_stream(s.cuda_stream)
        d.step_async(3)
        d.sync()
        t1 = time_steps(d, s, args.batched_steps, torch)
        perm[f"T{T}L{L}"] = t1 * 1e3
        seq += n * t1
        del d
    mixed["one_by_one_fp64"] = {"sypd": 96 * sypd(seq), "ms_per_step": seq * 1e3, "ms_per_member_step": perm}
    # the same 96 members on the host cores: the CPU oracle's timing build, every member stepped with all
    # threads (one member of each configuration timed, 3 steps after 3 warm-up, times 32)
    cores, _ = host_cpu()
    cpu_seq, cpu_perm = 0.0, {}
    for T, L, n in cfg:
        t1 = oracle_step_time(args, cores, 3, trunc=T, nlev=L)
        cpu_perm[f"T{T}L{L}"] = t1 * 1e3
        cpu_seq += n * t1
    mixed["cpu_oracle"] = {"sypd": 96 * sypd(cpu_seq), "ms_per_step": cpu_seq * 1e3, "ms_per_member_step": cpu_perm,
                           "cores": cores, "kind": "port",
                           "sample": "3 steps of one member per configuration on all cores, times 32 members"}
    for name in ("fp64", "split", "fp64_branches", "split_branches"):
        mixed[name]["vs_one_by_one_fp64"] = mixed[name]["sypd"] / mixed["one_by_one_fp64"]["sypd"]
    out["mixed"] = mixed
    out["autotune"] = tunelog
    return out


def arm_config(args, nlon, nlat, world):
    """The workload both arms report (the reference arm runs the same configuration on the host)."""
    return {"workload": f"held_suarez_T{args.trunc}L{args.nlev}_dt1800_fp64", "members_per_gpu": 1,
            "grid": f"{nlon}x{nlat}", "l2": "flushed (256 MB write) before every timed step",
            "precision": "fp64", "parallelism": f"replicas x{world}"}


# ---------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import numpy as np
    import oracle.pyoracle as po
    from aeros_gb300.params import held_suarez_params
    cores, model = host_cpu()
    po.use_variant("fast")
    po.set_threads(cores)
    p = held_suarez_params(trunc=args.trunc, nlev=args.nlev)
    o = po.OracleDyn(p, nthreads=cores)
    s = po.OracleSHT(args.trunc)
    o.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(0)
    tg = s.synthesis(t) + rng.normal(0.0, 0.1, (o.nlev, o.nlat, o.nlon))
    o.set_state(vor, div, s.analysis(tg), lnps)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = (time.perf_counter() - t0) / args.steps
    v = sypd(dt)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "SYPD", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": arm_config(args, o.nlon, o.nlat, world),
            "cpu_baseline": {"value": v, "unit": "SYPD", "cores": cores, "kind": "port", "cpu_model": model,
                             "build": "oracle/aeros_oracle.cpp, g++ -O3 -ffp-contract=fast -funroll-loops -fopenmp",
                             "sample": f"{args.steps} oracle steps after {args.warmup} warm-up, OpenMP over "
                                       f"levels and columns"},
            "e2e": {"value": v, "unit": "SYPD", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def host_cpu():
    """Host core count and CPU model (lscpu), for the CPU-baseline record."""
    import subprocess
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return os.cpu_count() or 1, model


def oracle_step_time(args, threads, nsteps, trunc=None, nlev=None):
    """Seconds per Held-Suarez step of the CPU oracle's timing build on `threads`
    OpenMP threads, from the config's initial state after 3 warm-up steps."""
    import numpy as np
    import oracle.pyoracle as po
    from aeros_gb300.params import held_suarez_params
    trunc = trunc or args.trunc
    nlev = nlev or args.nlev
    po.use_variant("fast")
    po.set_threads(threads)
    p = held_suarez_params(trunc=trunc, nlev=nlev)
    o = po.OracleDyn(p, nthreads=threads)
    s = po.OracleSHT(trunc)
    o.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(0)
    o.set_state(vor, div, s.analysis(s.synthesis(t) + rng.normal(0, 0.1, (o.nlev, o.nlat, o.nlon))), lnps)
    o.step(3)
    t0 = time.perf_counter()
    o.step(nsteps)
    return (time.perf_counter() - t0) / nsteps


def cpu_baseline_sample(args):
    """The oracle (CPU restatement of the reference's algorithm, timing build:
    -O3, fused multiply-adds, per-thread column scratch) timed on this host's
    cores at all threads and at one thread, bounded samples."""
    cores, model = host_cpu()
    n = args.cpu_steps
    dt = oracle_step_time(args, cores, n)
    n1 = max(3, n // 6)
    dt1 = oracle_step_time(args, 1, n1)
    return {"value": sypd(dt), "unit": "SYPD", "cores": cores, "kind": "port", "cpu_model": model,
            "ms_per_step": dt * 1e3,
            "one_thread": {"value": sypd(dt1), "unit": "SYPD", "ms_per_step": dt1 * 1e3, "steps": n1},
            "build": "oracle/aeros_oracle.cpp, g++ -O3 -ffp-contract=fast -funroll-loops -fopenmp",
            "sample": f"{n} Held-Suarez T{args.trunc}L{args.nlev} steps of the CPU oracle after 3 warm-up on "
                      f"{cores} OpenMP threads (levels and columns), and {n1} steps on one thread"}


# ---------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, local):
    import numpy as np
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(0)
    from __graft_entry__ import build
    if local == 0:
        build()
    if world > 1:
        dist.barrier()
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300.spectral import AerosSHT

    p = held_suarez_params(trunc=args.trunc, nlev=args.nlev)
    dyn = AerosDyn(p)
    sht = AerosSHT(args.trunc, batch_max=args.nlev)
    st = initial_state(dyn, sht, seed=rank)
    dyn.set_state(*st)
    stream = torch.cuda.Stream()
    dyn.set_stream(stream.cuda_stream)
    # launch shapes for this GPU and workload, chosen outside the timed region
    tune = None if args.no_tune else dyn.autotune(reps=5)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    dyn.step_async(max(args.warmup, 3))
    dyn.sync()
    torch.cuda.synchronize()
    K = args.steps
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = dyn.launch_count()
    with torch.cuda.stream(stream):
        for i in range(K):
            flush.fill_(i & 0xFF)           # L2 flush, outside the event pair
            ev0[i].record(stream)
            dyn.step_async(1)
            ev1[i].record(stream)
    dyn.sync()
    torch.cuda.synchronize()
    launches = dyn.launch_count() - n0
    t_gpu = sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)) / 1e3 / K
    # steady state with the state resident in L2 (no flush), for reference
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        dyn.step_async(K)
        e1.record(stream)
    dyn.sync()
    torch.cuda.synchronize()
    t_warm = e0.elapsed_time(e1) / 1e3 / K
    clk = clocks.stop()
    if world > 1:
        t_gpu = reduce_time(t_gpu, world, backend="nccl")
        dist.barrier()

    # per-kernel durations (events between the step's launches), averaged
    prof = {}
    for _ in range(5):
        for name, ms in dyn.profile_step():
            prof.setdefault(name, []).append(ms)
    prof = {k: sum(v) / len(v) for k, v in prof.items()}
    dom = max(prof, key=prof.get)
    work = kernel_work(args.trunc, dyn.nlat, dyn.nlon, sht.nlm, args.nlev)
    kind, amount = work.get(dom, ("flops", 0.0))
    hbm_gbs, bf16_tf, peak_src = measured_peaks()
    fp64_tf = fp64_peak_tflops(torch)
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"dram_traffic_T{args.trunc}L{args.nlev}.txt")
    if os.path.exists(tp):
        with open(tp) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and parts[0] == dom:
                    traffic = float(parts[1])
    if kind == "flops":
        achieved = amount / (prof[dom] / 1e3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_tf, "unit": "TFLOP/s",
                "frac": achieved / fp64_tf, "traffic": traffic, "kernel": dom,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)",
                "work_per_launch": amount}
        if dom == "column":
            # the grid bytes the column kernel must move, against the HBM peak (not what bounds it)
            gb = 8.0 * dyn.nlon * dyn.nlat * ((7 * args.nlev + 3) + (4 * args.nlev + 1))
            roof["hbm"] = {"bytes_per_launch": gb, "achieved_GBs": gb / (prof[dom] / 1e3) / 1e9,
                           "frac": gb / (prof[dom] / 1e3) / 1e9 / hbm_gbs}
    else:
        achieved = amount / (prof[dom] / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_gbs, "unit": "GB/s",
                "frac": achieved / hbm_gbs, "traffic": traffic, "kernel": dom,
                "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})", "work_per_launch": amount}
    # the same fraction for every kernel of the step (the dominant one changes with small timing shifts)
    per_kernel = {}
    for name, ms in prof.items():
        k_kind, k_amount = work.get(name, ("flops", 0.0))
        if k_kind == "flops":
            a = k_amount / (ms / 1e3) / 1e12
            per_kernel[name] = {"ms": ms, "achieved": a, "unit": "TFLOP/s", "frac": a / fp64_tf}
        else:
            a = k_amount / (ms / 1e3) / 1e9
            per_kernel[name] = {"ms": ms, "achieved": a, "unit": "GB/s", "frac": a / hbm_gbs}
    roof["per_kernel"] = per_kernel

    # e2e through the C-ABI with pinned host buffers
    e2e = None
    if True:
        s_now = [x.copy() for x in dyn.get_state()]
        s_old = [x.copy() for x in dyn.get_old_state()]
        nstep = dyn.counters()[0]
        def pinned(a):
            t = torch.empty(a.shape, dtype=torch.complex128, pin_memory=True)
            t.numpy()[...] = a
            return t.numpy()
        # one time level packed vor | div | temp | lnps, as aeros_dyn_step_packed takes it
        hn = pinned(dyn.pack(*s_now))
        ho = pinned(dyn.pack(*s_old))
        hout = pinned(dyn.pack(*s_now))
        hold = pinned(dyn.pack(*s_old))
        ne = max(20, min(K, 200))
        for _ in range(3):
            dyn.step_packed(hn, ho, nstep, 1, hout, hold)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ne):
            dyn.step_packed(hn, ho, nstep, 1, hout, hold)
        t_e2e = (time.perf_counter() - t0) / ne
        sbytes = hn.nbytes
        e2e = {"value": sypd(t_e2e) * world, "unit": "SYPD", "h2d_bytes_per_step": 2 * sbytes,
               "d2h_bytes_per_step": 2 * sbytes, "ms_per_step": t_e2e * 1e3,
               "path": "aeros_dyn_step_packed (X^n and X^(n-1) in, one step, both new time levels out) with "
                       "pinned host buffers: one graph launch and one synchronisation per step"}

    # split-precision form at the same workload, and its distance from the FP64 path
    split = None
    if not args.no_split:
        split = split_form(args, sht, dyn, flush, torch)
    batched = None
    if not args.no_batched:
        batched = batched_form(args, torch, t_gpu)

    adjoint = None
    if not args.no_adjoint and rank == 0:
        adjoint = adjoint_form(args)
    sweep = None
    if not args.no_sweep and rank == 0:
        sweep = transform_sweep(args, torch)
    transport = None
    if not args.no_transport and rank == 0:
        transport = transport_form(args, torch)

    cpu = cpu_baseline_sample(args) if (rank == 0 and world == 1) else None
    if rank == 0:
        line = {"metric": METRIC, "value": sypd(t_gpu) * world, "unit": "SYPD", "n_gpus": world, "steps": K,
                "warmup": args.warmup, "ms_per_step": t_gpu * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": arm_config(args, dyn.nlon, dyn.nlat, world),
                "ms_per_step_l2_resident": t_warm * 1e3,
                "launch_shapes": None if tune is None else {"ms_before": tune[0], "ms_after": tune[1],
                                                            "shapes": tune[2]},
                "sypd_l2_resident": sypd(t_warm) * world,
                "e2e": e2e, "roofline": roof, "kernels_ms": prof, "cpu_baseline": cpu,
                "split_precision": split, "batched": batched, "adjoint": adjoint, "transform_sweep": sweep,
                "transport": transport,
                "clocks": clk, "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    rank, world, local = rank_info()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
