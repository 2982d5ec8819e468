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
    return ap.parse_args()


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
def kernel_work(T, nlat, nlon, nlm, nlev):
    """Algorithmic work per launch of each step kernel at one member:
    flops for the contractions and FFTs (FP64), bytes for the memory-bound ones.
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
        "column": ("bytes", 8.0 * ng * ((7 * nlev + 3) + (4 * nlev + 1))),
        "fourier_anal": ("flops", fft * nlat * (4 * nlev + 1)),
        "legendre_anal": ("flops", F_leg * (6 * nlev + 1)),
        "spectral": ("bytes", 5.0 * st_bytes),
        "mass_rows": ("flops", F_leg + 2 * fft * 1.0),
        "mass_fix": ("bytes", 8.0 * nlat),
    }


def initial_state(dyn, sht, seed):
    """Held-Suarez start: rest, T = 264 K, ps = 1000 hPa, N(0, 0.1^2) K on grid T."""
    import numpy as np
    dyn.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = dyn.get_state()
    rng = np.random.default_rng(seed)
    tg = sht.synthesis(t) + rng.normal(0.0, 0.1, (dyn.nlev, dyn.nlat, dyn.nlon))
    return vor, div, sht.analysis(tg), lnps


# ---------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import numpy as np
    from oracle.pyoracle import OracleDyn, OracleSHT, set_threads
    from aeros_gb300.params import held_suarez_params
    cores = os.cpu_count() or 1
    set_threads(cores)
    p = held_suarez_params(trunc=args.trunc, nlev=args.nlev)
    o = OracleDyn(p, nthreads=cores)
    s = OracleSHT(args.trunc)
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
            "config": {"workload": f"held_suarez_T{args.trunc}L{args.nlev}_dt1800", "members": 1,
                       "grid": f"{o.nlon}x{o.nlat}"},
            "cpu_baseline": {"value": v, "unit": "SYPD", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} oracle steps after {args.warmup} warm-up, OpenMP over levels"},
            "e2e": {"value": v, "unit": "SYPD", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_sample(args):
    """The oracle (CPU restatement) timed on this host's cores, bounded sample."""
    import numpy as np
    from oracle.pyoracle import OracleDyn, OracleSHT, set_threads
    from aeros_gb300.params import held_suarez_params
    cores = os.cpu_count() or 1
    set_threads(cores)
    p = held_suarez_params(trunc=args.trunc, nlev=args.nlev)
    o = OracleDyn(p, nthreads=cores)
    s = OracleSHT(args.trunc)
    o.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(0)
    o.set_state(vor, div, s.analysis(s.synthesis(t) + rng.normal(0, 0.1, (o.nlev, o.nlat, o.nlon))), lnps)
    o.step(3)
    n = args.cpu_steps
    t0 = time.perf_counter()
    o.step(n)
    dt = (time.perf_counter() - t0) / n
    return {"value": sypd(dt), "unit": "SYPD", "cores": cores, "kind": "port",
            "ms_per_step": dt * 1e3,
            "sample": f"{n} Held-Suarez T{args.trunc}L{args.nlev} steps of the CPU oracle after 3 warm-up, "
                      f"{cores} OpenMP threads"}


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
    tp = os.path.join(ROOT, "profiles", f"{dom}_T{args.trunc}L{args.nlev}.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    if kind == "flops":
        achieved = amount / (prof[dom] / 1e3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_tf, "unit": "TFLOP/s",
                "frac": achieved / fp64_tf, "traffic": traffic, "kernel": dom,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)",
                "work_per_launch": amount}
    else:
        achieved = amount / (prof[dom] / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_gbs, "unit": "GB/s",
                "frac": achieved / hbm_gbs, "traffic": traffic, "kernel": dom,
                "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})", "work_per_launch": amount}

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
        hn = [pinned(x) for x in s_now]
        ho = [pinned(x) for x in s_old]
        hout = [pinned(x) for x in s_now]
        ne = max(20, min(K, 200))
        for _ in range(3):
            dyn.set_state(*hn); dyn.set_old_state(*ho, nstep=nstep); dyn.step(1); dyn.get_state(out=hout)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ne):
            dyn.set_state(*hn)
            dyn.set_old_state(*ho, nstep=nstep)
            dyn.step(1)
            dyn.get_state(out=hout)
        t_e2e = (time.perf_counter() - t0) / ne
        sbytes = sum(x.nbytes for x in hn)
        e2e = {"value": sypd(t_e2e) * world, "unit": "SYPD", "h2d_bytes_per_step": 2 * sbytes,
               "d2h_bytes_per_step": sbytes, "ms_per_step": t_e2e * 1e3,
               "path": "aeros_dyn_set_state/set_old_state/step/get_state with pinned host buffers"}

    cpu = cpu_baseline_sample(args) if (rank == 0 and world == 1) else None
    if rank == 0:
        line = {"metric": METRIC, "value": sypd(t_gpu) * world, "unit": "SYPD", "n_gpus": world, "steps": K,
                "warmup": args.warmup, "ms_per_step": t_gpu * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"held_suarez_T{args.trunc}L{args.nlev}_dt1800_fp64", "members_per_gpu": 1,
                           "grid": f"{dyn.nlon}x{dyn.nlat}", "l2": "flushed (256 MB write) before every timed step",
                           "precision": "fp64", "parallelism": f"replicas x{world}"},
                "ms_per_step_l2_resident": t_warm * 1e3,
                "sypd_l2_resident": sypd(t_warm) * world,
                "e2e": e2e, "roofline": roof, "kernels_ms": prof, "cpu_baseline": cpu,
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
