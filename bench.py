"""Benchmark of the GB300 D2Q9 BGK step (one JSON line on stdout).

Workload: lid-driven cavity 4096 x 4096, Re = 10000, U = 0.1, nu = 0.04096 (the reference's GPU
benchmark input UTIL/bgk.gpu.input), FP32 storage and arithmetic, fused ping-pong scheme.
A bench "step" is one lattice time step over the whole 4096^2 domain; the metric is GLUPS
(lx * ly * steps / time / 1e9, interior nodes, as SRC/finalize.F90:60-61 counts Mlups).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With N > 1 (torchrun) every rank advances its own cavity (independent domains, no exchange):
weak scaling, value = sum over ranks.  `--impl reference` times the CPU restatement of the
reference step (the oracle) on this machine's host cores for the same workload.

The line also carries the end-to-end figure (host buffers through the C ABI), the roofline of
the step kernel, the CPU baseline, the clocks seen while timing, `variants` (AA, FP16, BF16,
FP64, MIXED2, the two-pass form, LES) and `forms` (the 16-bit precision case, the 96-cavity
batch, the serving request stream).

  python bench.py --profile <scheme>_<storage> [--size n] [--tile c] [--prefetch p] [--les]
  python bench.py --profile batch_<storage> [--cases n]

run one small case and print its device time per step (the commands of the ncu summaries).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LX = LY = 4096
SVISC, U0 = 0.04096, 0.1
BYTES_PER_CELL = {"f32": 72, "f64": 144, "f16": 36, "bf16": 36}
WORKLOAD = "lid-driven cavity 4096x4096, Re=10000, U=0.1 (UTIL/bgk.gpu.input), FP32, fused ping-pong"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_ops_from_profiles(kernel_key):
    """FP64 instructions per cell of an FP64 collision kernel (profiles/fp64_ops_per_cell.txt)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "fp64_ops_per_cell.txt")):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel_key:
                return float(parts[1])
    except OSError:
        pass
    return None


def traffic_from_profiles(kernel_key):
    """DRAM bytes per launch recorded from an ncu capture (profiles/dram_traffic.txt)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel_key:
                return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples (every 50 ms) of SM clock and throttle reasons while the GPU works:
    started before the autotuner and stopped after the end-to-end runs, so that the record covers
    the timed region even when that region is a few milliseconds long."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev, period_ms=50):
        self.dev = dev
        self.period_ms = period_ms
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def __enter__(self):
        return self.start()

    def __exit__(self, *a):
        self.stop()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def summary(self):
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
                pw.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(pw), "period_ms": self.period_ms,
                "window": "autotune, warm-up, timed steps and end-to-end runs of the headline case"}


def free_port():
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def spawn_ranks(n, argv, script=None, timeout=3600):
    """One process per GPU when bench.py is started without torchrun: rank r runs `script argv`
    with RANK, LOCAL_RANK, WORLD_SIZE and MASTER_ADDR/PORT set (gloo carries the timing barrier
    and the max over ranks).  Rank 0's stdout is forwarded; returns the worst exit code."""
    script = script or os.path.abspath(__file__)
    port = free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, script] + list(argv), env=env,
                                      stdout=subprocess.PIPE if r == 0 else subprocess.DEVNULL, text=True))
    out, _ = procs[0].communicate(timeout=timeout)
    sys.stdout.write(out)
    sys.stdout.flush()
    rcs = [procs[0].returncode] + [p.wait(timeout=timeout) for p in procs[1:]]
    return next((rc for rc in rcs if rc != 0), 0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, dist=None):
    """Max of a per-rank time over all ranks (the job ends when the slowest rank ends)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_glups(cells_per_rank, steps, seconds, world):
    """Whole-job throughput: every rank advances its own domain (weak scaling)."""
    return world * cells_per_rank * steps / seconds / 1e9


def bench_config(world):
    """`config` of the JSON line, the same for both arms (tuning choices go elsewhere)."""
    return {"workload": WORKLOAD, "lx": LX, "ly": LY, "scheme": "pingpong", "storage": "f32",
            "l2": "inputs larger than L2: 1.21 GB of populations per step",
            "parallelism": f"{world} independent cavities, one per GPU" if world > 1 else "single domain"}


def cpu_reference(steps_budget_s=15.0, max_steps=None):
    """Time the oracle's threaded fused step on the host cores (bounded sample of the workload)."""
    from oracle import oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    o = orc.Oracle(LX, LY, prec=orc.SINGLE, tcase=orc.LDC, svisc=SVISC, u0=U0)
    o.step(1, threads=threads)  # warm-up (page in)
    n, t0 = 0, time.perf_counter()
    while True:
        o.step(1, threads=threads)
        n += 1
        el = time.perf_counter() - t0
        if el > steps_budget_s or (max_steps and n >= max_steps):
            break
    glups = LX * LY * n / el / 1e9
    o.close()
    return {"value": glups, "unit": "GLUPS", "cores": threads, "kind": "port",
            "sample": f"{n} fused steps of the 4096^2 FP32 cavity on {threads} threads ({el:.1f} s), "
                      "oracle/bgk_oracle.c (C restatement of SRC/col_MC.F90 + SRC/bcond.driven.F90)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    # a bounded sample: 5 s per 1000 requested steps, between 5 s and 60 s of host time
    cb = cpu_reference(steps_budget_s=min(60.0, max(5.0, 5.0 * args.steps / 1000)), max_steps=max(args.steps, 3))
    line = {"metric": "GLUPS", "value": cb["value"], "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": LX * LY / (cb["value"] * 1e9) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """Small case for ncu captures (or a quick timing of one tile shape): warm-up steps, then
    `--steps` device-timed steps; prints one tag line with the time per step."""
    import bgk2d_gpu_gb300 as bgk
    scheme, storage = args.profile.split("_")
    compute = args.compute or ("f64" if storage == "f64" else "f32")
    if scheme == "advance":  # host transfers: bgk_advance_host against upload + steps + download
        return run_profile_advance(args, storage, compute)
    if scheme == "batch":  # the first --cases cavities of the 96-cavity batch, one launch per step
        cases = cfg3_cases()[:args.cases]
        cells = sum(n * n for n, _, _ in cases)
        solvers = [bgk.Solver(n, n, tcase="LDC", svisc=u * n / re, u0=u, storage=storage, compute=compute)
                   for n, re, u in cases]
        with bgk.Batch(storage, compute) as b:
            for sv in solvers:
                b.add(sv)
            b.set_config(args.tile if args.tile >= 0 else 2, 0, 32)
            b.set_prefetch(args.prefetch)
            b.step(args.warmup)
            b.sync()
            ms = b.step_timed(args.steps)
        for sv in solvers:
            sv.close()
        per = ms / args.steps
        print(f"profile run {args.profile} {len(cases)} cavities ({cells} cells) tile={args.tile} "
              f"prefetch={args.prefetch} warmup={args.warmup} steps={args.steps} "
              f"ms/step={per:.4f} GLUPS={cells / (per * 1e-3) / 1e9:.2f}")
        return 0
    with bgk.Solver(args.size, args.size, tcase="LDC", svisc=SVISC * args.size / LX, u0=U0, storage=storage,
                    compute=compute, scheme=scheme, les=args.les) as s:
        if args.tile >= 0:
            s.set_tile(args.tile)
        s.set_prefetch(args.prefetch)
        s.step(args.warmup)
        s.sync()
        ms = s.step_timed(args.steps)
    per = ms / args.steps
    print(f"profile run {args.profile}{'_les' if args.les else ''} compute={compute} {args.size}^2 tile={args.tile} prefetch={args.prefetch} "
          f"warmup={args.warmup} steps={args.steps} "
          f"ms/step={per:.4f} GLUPS={args.size * args.size / (per * 1e-3) / 1e9:.2f}")
    return 0


def run_profile_advance(args, storage, compute):
    """--profile advance_<storage> --size n --steps K: the end-to-end call on page-locked host
    planes (rest state), median of five runs each: bgk_advance_host (pipelined), the three calls in
    sequence, and the upload and the download alone.  BGK_PIPE_ROWS sets the band height of the
    pipelined call."""
    import torch
    import bgk2d_gpu_gb300 as bgk
    L = bgk.load()
    n, K = args.size, args.steps
    tdt = torch.float64 if storage == "f64" else torch.float32
    with bgk.Solver(n, n, tcase="LDC", svisc=SVISC * n / LX, u0=U0, storage=storage, compute=compute) as s:
        s.tune(10)
        host = torch.zeros((9, n + 2, n + 2), dtype=tdt, pin_memory=True)
        out = torch.empty_like(host).pin_memory()
        pi, po = s._host_ptrs(host), s._host_ptrs(out)
        s.step(max(args.warmup, 65))
        s.sync()

        def med(fn, k=5):
            ts = []
            for _ in range(k):
                t0 = time.perf_counter()
                if fn():
                    raise RuntimeError("transfer call failed")
                ts.append(time.perf_counter() - t0)
            return sorted(ts)[k // 2] * 1e3
        adv = med(lambda: L.bgk_advance_host(s._h, pi, po, n + 2, K))
        seq = med(lambda: L.bgk_upload(s._h, pi, n + 2) | L.bgk_step(s._h, K) | L.bgk_download(s._h, po, n + 2))
        up = med(lambda: L.bgk_upload(s._h, pi, n + 2))
        dn = med(lambda: L.bgk_download(s._h, po, n + 2))
    nbytes = host.numel() * host.element_size()
    print(f"profile run advance_{storage} {n}^2 K={K}: advance_host {adv:.2f} ms ({n * n * K / adv / 1e6:.1f} GLUPS), "
          f"upload+step+download {seq:.2f} ms ({n * n * K / seq / 1e6:.1f} GLUPS), upload {up:.2f} ms "
          f"({nbytes / up / 1e6:.1f} GB/s), download {dn:.2f} ms ({nbytes / dn / 1e6:.1f} GB/s)")
    return 0


def measure_variant(bgk, storage, scheme, steps, warmup, dev, tune=True, les=False, compute=None, **kw):
    compute = compute or ("f64" if storage == "f64" else "f32")
    with bgk.Solver(LX, LY, tcase="LDC", svisc=SVISC, u0=U0, storage=storage, compute=compute, scheme=scheme,
                    device=dev, les=les, **kw) as s:
        cfg = s.tune(4 if compute == "f64" else 10)[0] if tune else None
        pf = s.prefetch()
        s.step(warmup)
        s.sync()
        ms = s.step_timed(steps)
    glups = LX * LY * steps / (ms * 1e-3) / 1e9
    return glups, ms / steps, cfg, pf


# ---------------------------------------------------------------------------------------------
# Other forms of the path, reported beside the headline (each bounded in time)
# ---------------------------------------------------------------------------------------------
def bench_precision(bgk, dev, n=2048, steps=10000):
    """Taylor-Green 2048^2, U0 = 0.02, tau = 0.6, 10000 steps: 16-bit storage against an FP64 run,
    and the FP64 decay of the vortex mode against exp(-nu (kx^2 + ky^2) t).  The mode amplitude
    is the projection of (u, v) on the initial field, read at a whole number of periods of the
    2k acoustic wave that the equilibrium start excites (T = n sqrt(3) / 2), where the density
    modulation of u = j / rho returns to its initial phase."""
    import numpy as np
    tau, u0 = 0.6, 0.02
    nu = (tau - 0.5) / 3.0
    t_dec = int(round(int(steps / (n * np.sqrt(3) / 2)) * n * np.sqrt(3) / 2))

    def run(st):
        kw = dict(tcase="TGV", storage=st, omega=1.0 / tau, svisc=nu, u0=0.0, init="tgv", tgv_u0=u0, device=dev)
        # the faster scheme of the kind, each tuned on a separate copy so that the measured run
        # keeps its step count: at 2048^2 one 16-bit AA buffer (75 MB) stays in L2, the two
        # ping-pong buffers (151 MB) do not
        best = None
        for scheme in (("pingpong",) if st == "f64" else ("pingpong", "aa")):
            with bgk.Solver(n, n, scheme=scheme, **kw) as t:
                cfg, _ = t.tune(4 if st == "f64" else 8)
                pf = t.prefetch()
                t.step(8)
                t.sync()
                tm = t.step_timed(16 if st == "f64" else 200)
            if best is None or tm < best[0]:
                best = (tm, scheme, cfg, pf)
        _, scheme, cfg, pf = best
        with bgk.Solver(n, n, scheme=scheme, **kw) as s:
            s.set_tile(cfg)
            s.set_prefetch(pf)
            _, ui, vi = s.fields()
            ms = s.step_timed(t_dec)
            _, ud, vd = s.fields()
            ms += s.step_timed(steps - t_dec)
            _, u, v = s.fields()
        amp = float(np.sum(ud * ui + vd * vi) / np.sum(ui * ui + vi * vi))
        return u, v, ms, amp, scheme

    u64, v64, ms64, amp, _ = run("f64")
    k2 = 2 * (2 * np.pi / n) ** 2
    rate = -np.log(amp) / t_dec
    out = {"workload": f"Taylor-Green {n}x{n}, U0={u0}, tau={tau}, {steps} steps",
           "fp64_mode_decay_rate": rate, "analytic_rate": nu * k2, "decay_window_steps": t_dec,
           "fp64_decay_rate_rel_err": float(abs(rate / (nu * k2) - 1)),
           "fp64_GLUPS": round(n * n * steps / (ms64 * 1e-3) / 1e9, 3)}
    den = float(np.sqrt(np.sum(u64 ** 2 + v64 ** 2)))
    for st in ("f32", "f16", "bf16"):
        u, v, ms, a, scheme = run(st)
        err = float(np.sqrt(np.sum((u - u64) ** 2 + (v - v64) ** 2)) / den)
        out[st] = {"velocity_L2_vs_fp64": err, "GLUPS": round(n * n * steps / (ms * 1e-3) / 1e9, 3), "scheme": scheme,
                   "decay_rate_rel_err": float(abs(-np.log(a) / t_dec / (nu * k2) - 1))}
    for st in ("f16", "bf16"):
        out[st]["over_f32"] = round(out[st]["GLUPS"] / out["f32"]["GLUPS"], 3)
    return out


def bench_precision_ldc(bgk, dev, steps=2000):
    """The headline cavity (4096^2, Re = 10000, 2000 steps) in FP64, FP32, FP16 and BF16 storage:
    GLUPS of each, device-timed over the same run, and the velocity-field L2 error of each
    against the FP64 run, ||u - u64||_2 / ||u64||_2 over the interior."""
    import numpy as np

    def run(st):
        kw = dict(tcase="LDC", svisc=SVISC, u0=U0, storage=st, device=dev)
        with bgk.Solver(LX, LY, **kw) as t:  # tuned on a separate copy: the measured run keeps its step count
            cfg, _ = t.tune(4 if st == "f64" else 10)
            pf = t.prefetch()
        with bgk.Solver(LX, LY, **kw) as s:
            s.set_tile(cfg)
            s.set_prefetch(pf)
            ms = s.step_timed(steps)
            _, u, v = s.fields()
        return u, v, LX * LY * steps / (ms * 1e-3) / 1e9

    u64, v64, g64 = run("f64")
    den = float(np.sqrt(np.sum(u64 ** 2 + v64 ** 2)))
    out = {"workload": f"lid-driven cavity {LX}x{LY}, Re=10000, U=0.1, {steps} steps", "f64": {"GLUPS": round(g64, 3)}}
    for st in ("f32", "f16", "bf16"):
        u, v, g = run(st)
        out[st] = {"GLUPS": round(g, 3),
                   "velocity_L2_vs_fp64": float(np.sqrt(np.sum((u - u64) ** 2 + (v - v64) ** 2)) / den)}
    for st in ("f16", "bf16"):
        out[st]["over_f32"] = round(out[st]["GLUPS"] / out["f32"]["GLUPS"], 3)
    return out


def host_link(torch, host, out, dev):
    """Page-locked host <-> device copy rates of one 604 MB buffer by the copy engines
    (cudaMemcpyAsync through torch), each direction alone and both at once: the ceiling of the
    end-to-end transfers."""
    d = torch.empty(host.shape, dtype=host.dtype, device=f"cuda:{dev}")
    nbytes = host.numel() * host.element_size()
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(fn, reps=4):
        best = 1e30
        for r in range(reps):
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s1)
            fn()
            e1.record(s1)
            e1.synchronize()
            if r:
                best = min(best, e0.elapsed_time(e1))
        return best

    def h2d():
        with torch.cuda.stream(s1):
            d.copy_(host, non_blocking=True)

    def d2h():
        with torch.cuda.stream(s1):
            out.copy_(d, non_blocking=True)

    def both():
        half = host.shape[0] // 2
        ev = torch.cuda.Event()
        ev.record(s1)
        s2.wait_event(ev)
        with torch.cuda.stream(s1):
            d[:half].copy_(host[:half], non_blocking=True)
        with torch.cuda.stream(s2):
            out[half:].copy_(d[half:], non_blocking=True)
        ev2 = torch.cuda.Event()
        ev2.record(s2)
        s1.wait_event(ev2)

    t_up, t_dn = timed(h2d), timed(d2h)
    half_bytes = (host.shape[0] // 2) * host[0].numel() * host.element_size()
    rest_bytes = nbytes - half_bytes
    t_bi = timed(both)
    del d
    return {"h2d_GBps": round(nbytes / t_up / 1e6, 1), "d2h_GBps": round(nbytes / t_dn / 1e6, 1),
            "both_GBps": round((half_bytes + rest_bytes) / t_bi / 1e6, 1),
            "how": "pinned 604 MB buffer, cudaMemcpyAsync (torch copy_), best of 3, CUDA events"}


def cfg3_cases(seed=0, count=96):
    """96 lid-driven cavities: edge in {128, 192, ..., 1536}, Re log-uniform [100, 5000],
    lid speed uniform [0.05, 0.1], tau = 3 U N / Re + 1/2."""
    import numpy as np
    rng = np.random.default_rng(seed)
    edges = np.arange(128, 1537, 64)
    out = []
    for _ in range(count):
        n = int(rng.choice(edges))
        re = float(np.exp(rng.uniform(np.log(100), np.log(5000))))
        u = float(rng.uniform(0.05, 0.1))
        out.append((n, re, u))
    return out


def bench_batched(bgk, dev, steps=5000, seq_steps=1000):
    cases = cfg3_cases()
    cells = sum(n * n for n, _, _ in cases)
    solvers = [bgk.Solver(n, n, tcase="LDC", svisc=u * n / re, u0=u, device=dev) for n, re, u in cases]
    with bgk.Batch("f32", device=dev) as b:
        for s in solvers:
            b.add(s)
        tuned = b.tune(6)
        b.sync()
        l0 = b.launches()
        ms = b.step_timed(steps - tuned)
        launches = b.launches() - l0
        cfg = b.config()
    for s in solvers:
        s.close()
    batched = cells * (steps - tuned) / (ms * 1e-3) / 1e9
    # the same cases one at a time with the plain single-domain kernel
    t_seq = 0.0
    for n, re, u in cases:
        with bgk.Solver(n, n, tcase="LDC", svisc=u * n / re, u0=u, device=dev) as s:
            s.step(4)
            s.sync()
            t_seq += s.step_timed(seq_steps) * 1e-3
    seq = cells * seq_steps / t_seq / 1e9
    return {"workload": f"96 lid-driven cavities (seed 0), {cells} cells, FP32, {steps} steps each",
            "batched_GLUPS": round(batched, 3), "one_at_a_time_GLUPS": round(seq, 3),
            "speedup": round(batched / seq, 3), "tuned_config": {"tile": cfg[0], "blocks_per_sm": cfg[1],
                                                                  "graph_steps": cfg[2]},
            "autotune_steps": tuned, "launches": launches,
            "hbm_frac": round(72 * batched / peaks()[0], 4)}


def cfg4_stream(rate, count, seed=1, storages=("f32", "f16")):
    """Poisson arrivals of three case types (cavity, cylinder channel, Taylor-Green); each request
    stores its populations in one of `storages` (equally likely)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        kind = rng.choice(["ldc", "cylinder", "tgv"])
        storage = storages[min(int(rng.uniform() * len(storages)), len(storages) - 1)]
        if kind == "ldc":
            n = int(rng.choice(np.arange(128, 2049, 64)))
            re = float(np.exp(rng.uniform(np.log(100), np.log(min(10000, 5 * n)))))
            tol = 1e-7 if rng.uniform() < 0.5 else 0.0
            r = dict(kind="ldc", n=n, re=re, u=0.1, storage=storage, max_steps=2000, tol=tol, check_every=500)
        elif kind == "cylinder":
            d = int(rng.choice([32, 48, 64, 96]))
            r = dict(kind="cylinder", n=d, re=float(rng.uniform(60, 200)), u=0.05, storage=storage, max_steps=2000)
        else:
            n = int(rng.choice(np.arange(512, 2049, 128)))
            r = dict(kind="tgv", n=n, re=float(rng.uniform(100, 1000)), u=0.02, storage=storage, max_steps=2000)
        reqs.append((t, r))
    return reqs


def bench_serving(bgk, dev, rates=(10.0, 30.0, 100.0), count=120, storages=("f32", "f16")):
    out = []
    for rate in rates:
        stream = cfg4_stream(rate, count, storages=storages)
        with bgk.Server(max_slots=64, chunk_steps=200, device=dev) as srv:
            t0 = time.perf_counter()
            for t, r in stream:
                dt = t - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                srv.submit(**r)
            srv.drain(600)
            res = srv.poll()
            st = srv.stats()
        out.append({"rate_per_s": rate, "storages": list(storages), "requests": count, "completed": st["completed"],
                    "failed": st["failed"],
                    "GLUPS": round(st["glups"], 3), "p50_s": round(st["p50_s"], 4), "p99_s": round(st["p99_s"], 4),
                    "mean_queue_s": round(st["mean_queue_s"], 4), "peak_resident": st["peak_resident"],
                    "launches": st["launches"], "rounds": st["rounds"],
                    "mean_round_steps": round(st["mean_round_steps"], 1),
                    "busy_frac": round(st["busy_s"] / st["wall_s"], 3) if st["wall_s"] else None,
                    "steps": int(sum(r["steps"] for r in res))})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the precision, batched and serving forms")
    ap.add_argument("--profile", default=None,
                    help="run only <scheme>_<storage> (e.g. pingpong_f32) on a --size^2 cavity, or batch_<storage> "
                         "on --cases cavities of the 96-cavity batch, for ncu")
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--tile", type=int, default=-1, help="tile configuration for --profile")
    ap.add_argument("--prefetch", type=int, default=0, help="L2 prefetch distance in blocks for --profile")
    ap.add_argument("--les", action="store_true", help="Smagorinsky collision for --profile")
    ap.add_argument("--compute", default=None, help="collision kind for --profile (f64 with f32 storage: MIXED2)")
    ap.add_argument("--cases", type=int, default=24, help="cavities of the batch for --profile batch_<storage>")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ and not args.profile:
        # started without torchrun: one process per GPU, launched here
        return spawn_ranks(args.gpus, sys.argv[1:])
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)

    rank, world, local = dist_env()
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if torch.cuda.device_count() < world:
            raise RuntimeError(f"{world} ranks but {torch.cuda.device_count()} visible GPUs")
    torch.cuda.set_device(local)
    import bgk2d_gpu_gb300 as bgk
    L = bgk.load()
    peak, peak_kind = peaks()
    clk = ClockSampler(local).start()

    # ---- device-timed value: K steps from HBM-resident state --------------------------------
    s = bgk.Solver(LX, LY, tcase="LDC", svisc=SVISC, u0=U0, storage="f32", scheme="pingpong", device=local)
    tile_cfg, _ = s.tune(10)
    prefetch = s.prefetch()
    s.step(args.warmup)
    s.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = s.launches()
    ms = s.step_timed(args.steps)
    torch.cuda.synchronize()
    launches = s.launches() - n0
    ms = max_over_ranks(ms, dist)
    glups = job_glups(LX * LY, args.steps, ms * 1e-3, world)
    ms_step = ms / args.steps
    achieved = BYTES_PER_CELL["f32"] * LX * LY / (ms_step * 1e-3) / 1e9
    diag = s.diagno()

    # ---- end-to-end through the C ABI with host buffers --------------------------------------
    # bgk_advance_host: 9 page-locked host planes up, K steps, 9 planes down, one call
    npl = (LX + 2) * (LY + 2)
    host = torch.zeros((9, LY + 2, LX + 2), dtype=torch.float32, pin_memory=True)  # rest state f = w
    out = torch.empty_like(host).pin_memory()
    ptr_in = s._host_ptrs(host)
    ptr_out = s._host_ptrs(out)
    # one-time setup outside the timed region: the step graphs of both buffer parities
    s.step(32)
    s.step(1)
    s.step(32)
    s.sync()
    if L.bgk_advance_host(s._h, ptr_in, ptr_out, LX + 2, args.steps):
        raise RuntimeError("advance_host failed")  # warm-up of the call itself

    def timed_runs(fn, n=3):
        runs = []
        for _ in range(n):
            if dist:
                dist.barrier()
            n1 = s.launches()
            t0 = time.perf_counter()
            rc = fn()
            runs.append(time.perf_counter() - t0)
            if rc:
                raise RuntimeError("end-to-end call failed")
        return runs, s.launches() - n1

    runs, e2e_launches = timed_runs(lambda: L.bgk_advance_host(s._h, ptr_in, ptr_out, LX + 2, args.steps))
    e2e_s = max_over_ranks(sorted(runs)[1], dist)
    # the same through the three separate calls, for comparison
    seq, _ = timed_runs(lambda: L.bgk_upload(s._h, ptr_in, LX + 2) | L.bgk_step(s._h, args.steps) |
                        L.bgk_download(s._h, ptr_out, LX + 2))
    seq_s = max_over_ranks(sorted(seq)[1], dist)
    link = host_link(torch, host, out, local) if rank == 0 else None
    xfer_bytes = 2 * 9 * npl * 4
    e2e = {"value": job_glups(LX * LY, args.steps, e2e_s, world), "unit": "GLUPS",
           "h2d_bytes_per_step": 9 * npl * 4 / args.steps, "d2h_bytes_per_step": 9 * npl * 4 / args.steps,
           "timed": "bgk_advance_host: 9 pinned host planes up, K steps, 9 planes down (pipelined), median of 3 runs",
           "runs_ms": [round(1e3 * t, 2) for t in runs], "launches": e2e_launches,
           "sequential": {"value": round(job_glups(LX * LY, args.steps, seq_s, world), 3),
                          "timed": "bgk_upload + bgk_step(K) + bgk_download, median of 3 runs",
                          "runs_ms": [round(1e3 * t, 2) for t in seq]}}
    if link:
        e2e["host_link"] = link
        e2e["link_frac"] = round(xfer_bytes / e2e_s / 1e9 / link["both_GBps"], 3)
    s.close()
    clk.stop()

    variants = {}
    if not args.no_variants and rank == 0:
        vsteps = max(20, args.steps // 10)
        # the FP64 steps are bound by the FP64 pipe: its measured instruction rate is their roofline
        import ctypes
        pk = (ctypes.c_double * 3)()
        fp64_peak = float(sum(pk)) / 3 / 1e9 if L.bgk_peak_fp64(local, pk) == 0 else None
        # les_*: the Smagorinsky collision (SRC/col_MC.F90:178-248), cteS = 0.1; noshift_f32: whole
        # populations in the planes (the NOSHIFT build, SRC/col_MC.F90:70-75)
        for name, st, sch, les in (("pingpong_f32", "f32", "pingpong", False), ("aa_f32", "f32", "aa", False),
                                   ("pingpong_f16", "f16", "pingpong", False), ("aa_f16", "f16", "aa", False),
                                   ("pingpong_bf16", "bf16", "pingpong", False),
                                   ("pingpong_f64", "f64", "pingpong", False), ("aa_f64", "f64", "aa", False),
                                   ("original_f32", "f32", "original", False),
                                   ("les_f32", "f32", "pingpong", True), ("les_f16", "f16", "pingpong", True),
                                   ("noshift_f32", "f32", "pingpong", False),
                                   ("mixed2_f32", "f32", "pingpong", False)):
            # mixed2: FP32 storage with the FP64 collision of the reference's MIXED2 build
            cp = "f64" if name.startswith("mixed2") else None
            n = vsteps if st != "f64" and cp is None else max(10, vsteps // 4)
            g, msv, cfg, pf = measure_variant(bgk, st, sch, n, 5, local, les=les, compute=cp,
                                              noshift=name.startswith("noshift"))
            # the two-pass form moves every population twice per step (stream, then collide)
            bw = BYTES_PER_CELL[st] * (2 if sch == "original" else 1) * LX * LY / (msv * 1e-3) / 1e9
            variants[name] = {"GLUPS": round(g, 3), "ms_per_step": round(msv, 4), "algorithmic_GBps": round(bw, 1),
                              "hbm_frac": round(bw / peak, 4), "steps": n, "tile_cfg": cfg,
                              "prefetch_blocks": pf}
            if (st == "f64" or cp == "f64") and fp64_peak:
                ops = fp64_ops_from_profiles("pp_kernel_mixed2" if cp == "f64" and st == "f32" else "pp_kernel_f64")
                if ops:
                    variants[name]["fp64_pipe"] = {
                        "ops_per_cell": ops, "achieved_Gops": round(g * ops, 1), "peak_Gops": round(fp64_peak, 1),
                        "frac": round(g * ops / fp64_peak, 4),
                        "peak_source": "bgk_peak_fp64 (DFMA/DADD/DMUL chains, this run)",
                        "ops_source": "profiles/fp64_ops_per_cell.txt (ncu, ping-pong kernel)"}

    forms = {}
    if rank == 0 and not args.no_forms:
        forms["precision_ldc4096"] = bench_precision_ldc(bgk, local)
        forms["precision_tgv2048"] = bench_precision(bgk, local)
        forms["batched_96_cavities"] = bench_batched(bgk, local)
        forms["serving_poisson"] = bench_serving(bgk, local)
        forms["serving_poisson_f32"] = bench_serving(bgk, local, rates=(100.0,), storages=("f32",))

    cpu = None
    if rank == 0 and not args.no_cpu and world == 1:
        cpu = cpu_reference(steps_budget_s=12.0)

    if rank == 0:
        kt = traffic_from_profiles(f"pp_kernel_f32_ldc4096_t{tile_cfg}_pf{prefetch}")
        line = {
            "metric": "GLUPS", "value": round(glups, 3), "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (rest-state start, no dataset)",
            "config": bench_config(world),
        }
        p16 = forms.get("precision_ldc4096")
        if p16:  # the 16-bit storage form on the same cavity, up front so that a tail of the line keeps it
            line["f16_GLUPS"] = p16["f16"]["GLUPS"]
            line["f16_over_f32"] = p16["f16"]["over_f32"]
            line["f16_L2_vs_fp64"] = p16["f16"]["velocity_L2_vs_fp64"]
            line["bf16_over_f32"] = p16["bf16"]["over_f32"]
            line["bf16_L2_vs_fp64"] = p16["bf16"]["velocity_L2_vs_fp64"]
        line.update({
            "tuning": {"tile_cfg": tile_cfg, "prefetch_blocks": prefetch},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": kt, "peak_kind": peak_kind,
                         "traffic_source": "profiles/dram_traffic.txt, same tile configuration and prefetch"
                         if kt is not None else "no capture of this configuration",
                         "kernel": ("bgk::pp_staged_kernel<float,float,...> (tile config %d)" if tile_cfg >= 6 else
                                    "bgk::pp_kernel<float,float,...> (tile config %d)") % tile_cfg,
                         "bytes_per_cell": 72},
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "diagno": [float(x) for x in diag],
            "variants": variants,
            "forms": forms,
        })
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
