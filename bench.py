"""Benchmark: 3D channel Helmholtz round trips on one GB300.

Workload (the configuration the headline metric is quoted on): Fourier 256
(C2C, x) x Fourier 256 (R2C, y) x Chebyshev ShenDirichlet 257 (z),
alpha = k^2 + 1/(nu dt) with nu dt = 1e-3, RHS i.i.d. N(0, 1) in physical
space from seed 0.  One step = scalar product of the RHS (inner(v, f)) ->
batched Helmholtz solve (33,024 band systems, one per (kx, ky)) -> backward
transform.  The factorisation is set-up work (done once, as in shenfun).

Two arithmetic forms are measured on the same input: the plain form (all
FP64) and the mixed ("chosen") form (FP64 in and out: the length-256 Fourier
axes in 64-bit fixed point on the integer pipes, the Chebyshev axis as
split-BF16 contractions on the tensor cores, the banded solve in FP64).
``value`` is the mixed form's throughput when its error against the FP64
oracle is within 1e-10, else the plain form's.

Prints one JSON line.  ``--impl reference`` times the reference's CPU path
(its compiled Cython Helmholtz kernels when built in oracle/_ref, transforms
through scipy.fft standing in for FFTW) on the host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

NX, NY, NZ = 256, 256, 257
NU_DT = 1e-3
C_SHIFT = 1.0 / NU_DT
MIXED_TOL = 1e-10
METRIC = "Helmholtz solves/s (chosen vs plain FP64, rel err <=1e-10); p50/p99 latency"
WORKLOAD = ("3D channel Helmholtz round trip: Fourier 256 (C2C) x Fourier 256 (R2C) x "
            "Chebyshev ShenDirichlet 257, alpha=k^2+1/(nu*dt), nu*dt=1e-3, RHS N(0,1) seed 0")

# algorithmic bytes per launch (read + write of each array touched once)
R_BYTES = NX * NY * NZ * 8                      # physical real array
C_BYTES = NX * (NY // 2 + 1) * NZ * 16          # spectral complex array
F_BYTES = NX * (NY // 2 + 1) * (NZ - 2) * 8     # one factor array (cache layout)
STAGE_BYTES = {
    "z_scalar_product": 2 * R_BYTES,
    "y_r2c": R_BYTES + C_BYTES,
    "x_c2c_fwd": 2 * C_BYTES,
    "helmholtz_solve": 2 * C_BYTES + 4 * F_BYTES,
    "x_c2c_bwd": 2 * C_BYTES,
    "y_c2r": C_BYTES + R_BYTES,
    "z_backward": 2 * R_BYTES,
}
ROUNDTRIP_BYTES = sum(STAGE_BYTES.values())


def peaks(key="hbm_gbs", fallback=6800.0):
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d[key]), "measured"
    except Exception:
        return fallback, "fallback"


# the mixed form's Chebyshev-axis passes are split-BF16 contractions on the
# tensor cores: 28 digit products (7 digits, s + t <= 6) of a lines x NZ by
# NZ x NZ product, 2 flops per multiply-add (the tensor pipe's work; the
# roofline of the pass is still HBM bytes)
TC_PRODUCTS = 28
TC_FLOPS = TC_PRODUCTS * 2.0 * NX * NY * NZ * NZ
TC_STAGES = ("z_scalar_product", "z_backward")
# DRAM traffic per stage from the committed ncu summaries: a line
# "dram_bytes_per_pass: <bytes>" in the profile of the stage's kernels
TRAFFIC_PROFILES = {
    "mixed:z_scalar_product": "profiles/fused_contraction_256x256x257.md",
}


def profiled_traffic(key):
    """Per-pass DRAM bytes (read + write) recorded in the stage's committed
    ncu summary, or None when the stage has none."""
    import re
    path = TRAFFIC_PROFILES.get(key)
    if not path:
        return None
    try:
        m = re.search(r"dram_bytes_per_pass:\s*([0-9]+)", open(os.path.join(REPO, path)).read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_total_ms(tot_ms, dist=None, device="cpu"):
    """Replicas only (every rank solves its own copy, no data-path
    collective): the job's time is the slowest rank's."""
    if dist is None:
        return float(tot_ms)
    import torch
    t = torch.tensor([float(tot_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def agree(obj, dist=None):
    """Rank 0's decision on every rank (the error check runs on rank 0)."""
    if dist is None:
        return obj
    box = [obj]
    dist.broadcast_object_list(box, src=0)
    return box[0]


def setup_dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_leg(steps, warmup, threads):
    """Time the reference's CPU path on the full workload (a few solves)."""
    from oracle.cpu_baseline import HelmholtzRoundTrip, time_steps
    rt = HelmholtzRoundTrip(NX, NY, NZ, C_SHIFT, workers=threads)
    f = np.random.default_rng(0).standard_normal(rt.shape)
    ts = time_steps(rt, f, steps, warmup)
    return rt, ts


def run_reference(args):
    ws, rank, local = setup_dist()
    if rank != 0:
        return 0
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    rt, ts = cpu_leg(args.steps, args.warmup, threads)
    tot = float(sum(ts))
    val = len(ts) / tot
    solver = "reference Cython la.pyx" if rt.kind == "reference" else "numpy port"
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / len(ts), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "reference CPU path"},
        "latency_ms": {"p50": 1e3 * float(np.percentile(ts, 50)),
                       "p99": 1e3 * float(np.percentile(ts, 99))},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": rt.kind,
                         "sample": f"{len(ts)} full {NX}x{NY}x{NZ} round trips; transforms via "
                                   f"scipy.fft on {threads} threads (FFTW absent), Helmholtz "
                                   f"solve single-threaded ({solver}); factorisation excluded "
                                   f"({rt.setup_s:.2f} s)"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


class FormRun:
    """One arithmetic form of the workload: space, solver, arrays.  Forms:
    plain (all FP64), mixed (mixed transforms, FP64 direct banded solve) and
    mixed-refined (mixed transforms, FP32 banded solve refined by an FP64
    residual)."""

    def __init__(self, sg, form, f_np):
        self.form = form
        tform = "plain" if form == "plain" else "mixed"
        self.T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"),
                                              sg.FunctionSpace(NY, "F", dtype="d"),
                                              sg.FunctionSpace(NZ, "C", bc=(0, 0))), form=tform)
        u, self.v = sg.TrialFunction(self.T), sg.TestFunction(self.T)
        mats = sg.inner(self.v, -sg.div(sg.grad(u)) + C_SHIFT * u)
        if form == "mixed-refined":
            self.H = sg.chebyshev.la.Helmholtz(*mats, form="refined", residual="fp64")
        else:
            # the direct solve uses the FP64 factorisation cache: it measured
            # faster than its double-float variant (0.32 vs 0.51 ms)
            self.H = sg.chebyshev.la.Helmholtz(*mats, form="plain")
        self.sg = sg
        self.fj = sg.Array(self.T, buffer=f_np)
        self.f_hat = sg.Function(self.T)
        self.u_hat = sg.Function(self.T)
        self.uq = sg.Array(self.T)

    def step(self):
        self.sg.inner(self.v, self.fj, output_array=self.f_hat)
        self.H(self.f_hat, self.u_hat)
        self.T.backward(self.u_hat.v, self.uq.v)

    # our kernels per step: plain 7 (three axes each way + the solve); mixed
    # forms 9 (each Chebyshev pass is two: line scales, fused contraction)
    @property
    def launches_per_step(self):
        return 7 if self.form == "plain" else 9


def e2e_pipelined(torch, sg, run0, form, f_np, f_host, steps, st, nslots=3):
    """Solves/s through the public API with host buffers, `nslots` requests in
    flight: request i copies its RHS in (pinned H2D, its own stream), runs the
    round trip on the compute stream and copies its solution out (D2H, its own
    stream), while earlier requests' copy-outs and later requests' copy-ins
    overlap it.  Every step moves its full input and output across the host
    link."""
    slots = [run0] + [FormRun(sg, form, f_np) for _ in range(nslots - 1)]
    u_hosts = [torch.empty((NX, NY, NZ), dtype=torch.float64).pin_memory() for _ in slots]
    h2d, comp, d2h = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev = lambda: torch.cuda.Event()  # noqa: E731
    h_done = [ev() for _ in slots]
    c_done = [ev() for _ in slots]
    d_done = [ev() for _ in slots]

    def submit(i):
        k = i % nslots
        sl = slots[k]
        with torch.cuda.stream(h2d):
            if i >= nslots:
                h2d.wait_event(c_done[k])  # the slot's previous round trip read its RHS
            sl.fj.v.copy_(f_host, non_blocking=True)
            h_done[k].record(h2d)
        with torch.cuda.stream(comp):
            comp.wait_event(h_done[k])
            if i >= nslots:
                comp.wait_event(d_done[k])  # the slot's previous solution was copied out
            sl.step()
            c_done[k].record(comp)
        with torch.cuda.stream(d2h):
            d2h.wait_event(c_done[k])
            u_hosts[k].copy_(sl.uq.v, non_blocking=True)
            d_done[k].record(d2h)

    for i in range(2 * nslots):  # warm-up of every slot
        submit(i)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for s_ in (h2d, comp, d2h):
        s_.wait_stream(st)
    for i in range(steps):
        submit(i)
    for s_ in (h2d, comp, d2h):
        st.wait_stream(s_)
    b.record(st)
    b.synchronize()
    # the last solution arrived on the host and equals the resident result
    last = (steps - 1) % nslots
    assert torch.equal(u_hosts[last], slots[last].uq.v.cpu())
    return steps / (a.elapsed_time(b) / 1e3)


def time_steps_gpu(torch, fn, steps, flush, st):
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        evs[i][0].record(st)
        fn()
        evs[i][1].record(st)
    torch.cuda.synchronize()
    return np.array([a.elapsed_time(b) for a, b in evs])


def stage_times(torch, run, flush, st, reps=5):
    T, H = run.T, run.H
    sp = T.bases
    dev = run.fj.v.device
    wr = torch.empty((NX, NY, NZ), dtype=torch.float64, device=dev)
    wc = torch.empty((NX, NY // 2 + 1, NZ), dtype=torch.complex128, device=dev)
    wc2 = torch.empty_like(wc)
    stages = [
        ("z_scalar_product", lambda: sp[2].scalar_product(run.fj.v, wr, axis=2)),
        ("y_r2c", lambda: sp[1].scalar_product(wr, wc, axis=1)),
        ("x_c2c_fwd", lambda: sp[0].scalar_product(wc, wc2, axis=0)),
        ("helmholtz_solve", lambda: H(wc2, wc)),
        ("x_c2c_bwd", lambda: sp[0].backward(wc, wc2, axis=0)),
        ("y_c2r", lambda: sp[1].backward(wc2, wr, axis=1)),
        ("z_backward", lambda: sp[2].backward(wr, run.uq.v, axis=2)),
    ]
    out = {}
    for name, fn in stages:
        fn()
        torch.cuda.synchronize()
        out[name] = float(np.mean(time_steps_gpu(torch, fn, reps, flush, st)))
    return out


SERVE_SIZES = (32, 64, 128, 256, 512)
SERVE_SHIFTS = (0.1, 1.0, 10.0, 100.0, 1e3, 1e4)


def serving_leg(torch, nreq=10000, seed=5, form="mixed", fractions=(0.75, 0.5, 0.25), cache_gb=128,
                compare=2000):
    """Serving stream of `nreq` mixed 2D/3D Fourier x Chebyshev/Legendre
    Dirichlet Helmholtz requests: N per axis drawn log-uniformly from
    {32, 64, 128, 256, 512} (3D grids above 2^24 points redrawn), c drawn
    log-uniformly from {0.1, 1, 10, 100, 1e3, 1e4} (a population of fixed
    configurations, so that factorisations repeat), family 50/50, RHS N(0, 1)
    (two seeded arrays per grid shape, page-locked on the host; every request
    copies its RHS to the device).  One batching executor (graphs of batched
    steps, device factorisation cache of `cache_gb` GB and 24 GB of graph
    runners, each LRU) runs: all
    requests at once on a cold cache, all at once warm (saturation
    throughput C), then Poisson arrivals at each fraction of C (latency =
    completion - arrival).  The per-request executor (no batching) runs the
    first `compare` requests warm for comparison.  Solutions stay on the
    device."""
    import collections
    from shenfun_gb300 import serving as SV
    pool = SV.RhsPool(per_shape=2, seed=seed)
    runner_gb = 24
    budget = (cache_gb + runner_gb + 16) << 30

    def one(label, ex, rate, n):
        stream = SV.make_stream(n, seed=seed, rate=rate, sizes=SERVE_SIZES, shifts=SERVE_SHIFTS)
        h0, m0 = ex.hits, ex.misses
        b0 = collections.Counter(getattr(ex, "batch_sizes", {}))
        fin, elapsed = SV.run_stream(stream, ex, max_slots=256, mem_budget=budget, rhs=pool)
        torch.cuda.synchronize()
        done = [r for r in fin if r.state == SV.DONE]
        lat = np.array([r.latency for r in done])
        pts = sum(int(np.prod(r.N)) for r in done)
        res = {"run": label, "rate_req_per_s": rate, "requests": n, "completed": len(done),
               "failed": sum(r.state != SV.DONE for r in fin),
               "solves_per_s": len(done) / elapsed, "grid_points_per_s": pts / elapsed,
               "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
               "cache_hits": ex.hits - h0, "cache_misses": ex.misses - m0, "seconds": elapsed}
        if hasattr(ex, "batch_sizes"):
            bs = ex.batch_sizes - b0
            nb = sum(bs.values())
            res["batches"] = nb
            res["mean_batch"] = sum(k * v for k, v in bs.items()) / max(nb, 1)
            res["batch_size_hist"] = {str(k): v for k, v in sorted(bs.items())}
        return res

    ex = SV.BatchExecutor(nstreams=4, cache_budget=cache_gb << 30, keep_results=False, form=form,
                          runner_budget=runner_gb << 30)
    runs = [one("all at once, cold cache", ex, None, nreq), one("all at once, warm (saturation)", ex, None, nreq)]
    C = runs[-1]["solves_per_s"]
    for fr in fractions:
        runs.append(one(f"Poisson at {fr} x saturation", ex, fr * C, nreq))
    if ex.pool is not None:
        ex.pool.shutdown()
    del ex
    torch.cuda.empty_cache()
    ex1 = SV.GpuExecutor(nstreams=4, cache_budget=cache_gb << 30, keep_results=False, form=form)
    one("per-request executor, cold", ex1, None, compare)
    runs.append(one("per-request executor (no batching), all at once, warm", ex1, None, compare))
    return {"requests_per_run": nreq, "form": form, "sizes": list(SERVE_SIZES), "shifts": list(SERVE_SHIFTS),
            "cache_budget_gb": cache_gb, "rhs_host_gb": pool.nbytes / 1e9, "runs": runs}


def legendre_leg(torch, flush, st, N=512, lines=16384, reps=5):
    """Legendre ShenDirichlet lines of length N: coefficients
    c_k ~ U(-1, 1) (k + 1)^-2 (seed 0), backward then forward, in the plain
    FP64 form and in the mixed form (BF16 digit slices on the tensor cores).
    FP64-equivalent rate = 2 N^2 lines per direction / time; L2 flushed before
    every timed step."""
    from shenfun_gb300.legendre import LegendreShenDirichlet
    rng = np.random.default_rng(0)
    c = rng.uniform(-1, 1, (lines, N)) * (np.arange(N) + 1.0) ** -2
    c[:, -2:] = 0
    cd = torch.as_tensor(c, device="cuda")
    u = torch.empty_like(cd)
    c2 = torch.empty_like(cd)
    flops = 2.0 * N * N * lines
    out = {"N": N, "lines": lines, "data": "c_k ~ U(-1,1)(k+1)^-2, seed 0", "forms": {}}
    ref = None
    for form in ("plain", "mixed"):
        V = LegendreShenDirichlet(N, form=form)
        bwd = lambda: V.backward(cd, u, axis=1)  # noqa: E731
        fwd = lambda: V.forward(u, c2, axis=1)  # noqa: E731
        for _ in range(2):
            bwd()
            fwd()
        torch.cuda.synchronize()
        tb = float(np.mean(time_steps_gpu(torch, bwd, reps, flush, st)))
        tf = float(np.mean(time_steps_gpu(torch, fwd, reps, flush, st)))
        res = {"ms_backward": tb, "ms_forward": tf,
               "tflops_fp64_equiv_backward": flops / (tb * 1e-3) / 1e12,
               "tflops_fp64_equiv_forward": flops / (tf * 1e-3) / 1e12}
        if ref is None:
            ref = (u.clone(), c2.clone())
        else:
            res["rel_err_vs_plain"] = max(float(((u - ref[0]).abs().max() / ref[0].abs().max()).item()),
                                          float(((c2 - ref[1]).abs().max() / ref[1].abs().max()).item()))
        res["rel_err_roundtrip"] = float(((c2 - cd).abs().max() / cd.abs().max()).item())
        out["forms"][form] = res
    p_, m_ = out["forms"]["plain"], out["forms"]["mixed"]
    out["mixed_over_plain"] = (p_["ms_backward"] + p_["ms_forward"]) / (m_["ms_backward"] + m_["ms_forward"])
    return out


def legendre_cpu(N, lines_max=4096, budget_flop=3e8):
    """The reference's recursive Legendre transforms (compiled transforms.pyx
    when built, else the numpy restatement) on one host thread, on a sample
    of lines sized to about budget_flop multiply-adds per direction."""
    from oracle.cpu_baseline import LegendreLines, time_calls
    n = int(max(64, min(lines_max, budget_flop // (N * N))))
    L = LegendreLines(N, n)
    tb = float(np.median(time_calls(L.backward, 2)))
    tf = float(np.median(time_calls(L.forward, 2)))
    return {"kind": L.kind, "cores": 1, "sample_lines": n,
            "lines_per_s_backward": n / tb, "lines_per_s_forward": n / tf,
            "gflops_fp64_backward": 2.0 * N * N * n / tb / 1e9}


def legendre_sweep(torch, flush, st, Ns=(128, 256, 512, 1024), lines=(4096, 16384, 65536), reps=3):
    """The batched Legendre configuration: N in Ns x lines per launch, both
    forms (legendre_leg), and per N the reference's CPU transforms on a
    sample (lines/s on one thread; GPU/CPU ratio at the largest line count)."""
    out = []
    for N in Ns:
        cpu = legendre_cpu(N)
        for L in lines:
            r = legendre_leg(torch, flush, st, N=N, lines=L, reps=reps)
            m = r["forms"]["mixed"]
            r["lines_per_s_mixed"] = {"backward": L / (m["ms_backward"] * 1e-3),
                                      "forward": L / (m["ms_forward"] * 1e-3)}
            r["cpu_reference"] = cpu
            r["gpu_mixed_over_cpu"] = {
                "backward": r["lines_per_s_mixed"]["backward"] / cpu["lines_per_s_backward"],
                "forward": r["lines_per_s_mixed"]["forward"] / cpu["lines_per_s_forward"]}
            out.append(r)
    return out


def dlt_terms(N, total_lines, sample=8, seed=0, tol=1e-16):
    """Taylor terms the reference's fast backward Legendre transform takes at
    length N (legendre/dlt.py:166-186: term n is (-1)^.. dtheta^n / n! times a
    DCT (n even) or DST (n odd) of k^n x_k; the loop stops at the first term
    whose norm over the whole array is below 1e-16).  dtheta are the offsets
    between the Gauss-Legendre and Chebyshev-Gauss angles; x is a sample of
    lines with the legendre leg's coefficient decay, the norm scaled from the
    sample to total_lines lines."""
    import scipy.fft as F
    from shenfun_gb300.legendre import leggauss
    xl, _ = leggauss(N)
    dtheta = np.arccos(xl)[::-1] - (2 * np.arange(N) + 1) * np.pi / (2 * N)
    x = np.random.default_rng(seed).uniform(-1, 1, (sample, N)) * (np.arange(N) + 1.0) ** -2
    k = np.arange(N, dtype=float)
    y = np.ones(N)
    nfac = 1.0
    for n in range(1, 200):
        nfac *= n
        x = x * k
        y = y * dtheta
        h = (F.dct if n % 2 == 0 else F.dst)(x, type=3, axis=-1) / 2
        if np.linalg.norm(y * h) / nfac * np.sqrt(total_lines / sample) < tol:
            return n
    return 200


def dlt_bound_leg(torch, flush, st, Ns=(2048, 4096), lines=4096, reps=3):
    """The dense Legendre contraction against a lower bound of the reference's
    fast (DLT) transform at large N.  The DLT does one DCT plus one DCT or DST
    per Taylor term (dlt_terms), plus a leg2cheb conversion and O(N) scalings
    per term; the bound counts the DCT/DST passes only, each timed as this
    library's FP64 DCT-III pass over the same lines (a DST costs the same
    FFT), and leaves out leg2cheb altogether.  Beside it the dense Legendre
    backward and forward transforms (legendre_leg) on the same lines."""
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    out = []
    for N in Ns:
        x = torch.randn(lines, N, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        p = LinePlan(_lib.XF_DCT3, N, form=_lib.PLAIN_F64)
        run = lambda: p(x, y, 1)  # noqa: E731
        for _ in range(3):
            run()
        torch.cuda.synchronize()
        t_dct = float(np.mean(time_steps_gpu(torch, run, reps, flush, st)))
        terms = dlt_terms(N, lines)
        dense = legendre_leg(torch, flush, st, N=N, lines=lines, reps=reps)
        bound = (terms + 1) * t_dct
        out.append({"N": N, "lines": lines, "ms_dct_fp64": t_dct, "taylor_terms": terms,
                    "dlt_lower_bound_ms": bound,
                    "dense_ms": {f: {"backward": r["ms_backward"], "forward": r["ms_forward"]}
                                 for f, r in dense["forms"].items()},
                    "dense_mixed_rel_err_vs_plain": dense["forms"]["mixed"]["rel_err_vs_plain"],
                    "bound_over_dense_mixed": bound / dense["forms"]["mixed"]["ms_backward"]})
    return out


def biharmonic_leg(torch, flush, st, steps=10):
    """Fourier 128 (C2C) x Fourier 128 (R2C) x Chebyshev ShenBiharmonic 129,
    RHS f = lap^2 u of the manufactured u = sin(x) cos(y) (1 - z^2)^2
    sampled on the quadrature grid: scalar product -> biharmonic solve
    (8,320 banded + rank-2 semiseparable systems) -> backward, L2 flushed
    before every step; forms plain (FP64), mixed (mixed transforms, FP64
    direct solve) and mixed-refined (mixed transforms, FP32 solve refined by
    the FP64 residual); error of each form against u and against the plain
    form, correction counts of the refined solve.  The reference's CPU path
    on the same grid beside it (its LU_Biharmonic leaves the last even row
    unfactored when N - 4 is odd, as here, and its solve returns non-finite
    values: the CPU figure is a timing only)."""
    import shenfun_gb300 as sg
    Nx, Ny, Nz = 128, 128, 129
    x = 2 * np.pi * np.arange(Nx) / Nx
    y = 2 * np.pi * np.arange(Ny) / Ny
    z = np.cos(np.pi * (2 * np.arange(Nz) + 1) / (2 * Nz))
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    u_exact = np.sin(X) * np.cos(Y) * (1 - Z ** 2) ** 2
    f = np.sin(X) * np.cos(Y) * (44 - 56 * Z ** 2 + 4 * Z ** 4)
    out = {"workload": "Fourier 128 (C2C) x Fourier 128 (R2C) x Chebyshev ShenBiharmonic 129, "
                       "RHS lap^2 u, u = sin(x)cos(y)(1-z^2)^2"}
    ref = None
    ue = torch.as_tensor(u_exact, device="cuda")
    for form in ("plain", "mixed", "mixed-refined"):
        T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"), sg.FunctionSpace(Ny, "F", dtype="d"),
                                         sg.FunctionSpace(Nz, "C", bc=(0, 0, 0, 0))),
                                  form="plain" if form == "plain" else "mixed")
        u, v = sg.TrialFunction(T), sg.TestFunction(T)
        H = sg.chebyshev.la.Biharmonic(sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u))))),
                                       form="refined" if form == "mixed-refined" else "plain")
        fj = sg.Array(T, buffer=f)
        f_hat, u_hat, uq = sg.Function(T), sg.Function(T), sg.Array(T)

        def step():
            sg.inner(v, fj, output_array=f_hat)
            H(f_hat, u_hat)
            T.backward(u_hat.v, uq.v)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ms = float(np.mean(time_steps_gpu(torch, step, steps, flush, st)))
        res = {"ms_per_step": ms, "solves_per_s": 1e3 / ms,
               "rel_err_vs_exact": float(((uq.v - ue).abs().max() / ue.abs().max()).item())}
        # the solve alone
        H(f_hat, u_hat)
        torch.cuda.synchronize()
        res["solve_ms"] = float(np.mean(time_steps_gpu(torch, lambda: H(f_hat, u_hat), steps, flush, st)))
        if ref is None:
            ref = uq.v.clone()
        else:
            res["rel_err_vs_plain"] = float(((uq.v - ref).abs().max() / ref.abs().max()).item())
        if H.last_iterations is not None:
            it = H.last_iterations.cpu().numpy()
            res["corrections"] = {"max": int(it.max()), "mean": float(it.mean())}
        out[form] = res
    from oracle.cpu_baseline import BiharmonicRoundTrip, time_steps
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        rt = BiharmonicRoundTrip(Nx, Ny, Nz)
        ts = time_steps(rt, f, 3, 1)
        finite = bool(np.isfinite(rt.step(f)).all())
    out["cpu_baseline"] = {"value": len(ts) / float(sum(ts)), "unit": "solves/s", "cores": 1, "kind": rt.kind,
                           "sample": f"{len(ts)} full round trips on 1 host thread (scipy.fft for FFTW, "
                                     f"reference LU_Biharmonic/Biharmonic_Solve), factorisation excluded "
                                     f"({rt.setup_s:.2f} s)",
                           "output_finite": finite}
    return out


def refinement_leg(torch, flush, st, f_np, steps=10):
    """The channel grid's banded solves alone (33,024 systems of 255): FP64
    direct from the FP64 factor cache against FP32 sweeps (FP32 factor
    cache, half the bytes) refined by an FP64 or a double-float residual;
    error against the FP64 direct solution (which matches the oracle to
    1e-15), correction counts, time per solve (L2 flushed)."""
    import shenfun_gb300 as sg
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"), sg.FunctionSpace(NY, "F", dtype="d"),
                                     sg.FunctionSpace(NZ, "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    mats = sg.inner(v, -sg.div(sg.grad(u)) + C_SHIFT * u)
    f_hat = sg.inner(v, sg.Array(T, buffer=f_np))
    out = {"workload": "33,024 Chebyshev Dirichlet Helmholtz systems of 255 (the channel grid's solve)"}
    ref = None
    for name, kw in (("fp64_direct", {"form": "plain"}), ("fp32_refined_fp64_residual", {"form": "refined"}),
                     ("fp32_refined_df_residual", {"form": "refined", "residual": "df"})):
        H = sg.chebyshev.la.Helmholtz(*mats, **kw)
        uh = sg.Function(T)
        H(f_hat, uh)
        torch.cuda.synchronize()
        ms = float(np.mean(time_steps_gpu(torch, lambda: H(f_hat, uh), steps, flush, st)))
        res = {"solve_ms": ms, "factor_bytes": int(H._fac.numel() * H._fac.element_size())}
        if ref is None:
            ref = uh.v.clone()
        else:
            res["rel_err_vs_fp64_direct"] = float(((uh.v - ref)[..., :-2].abs().max() / ref.abs().max()).item())
            it = H.last_iterations.cpu().numpy()
            res["corrections"] = {"max": int(it.max()), "mean": float(it.mean())}
        out[name] = res
    return out


def neumann_leg(torch, flush, st, steps=10):
    """The Chebyshev boundary-condition row on the channel grid's sizes:
    Fourier 256 (C2C) x Fourier 256 (R2C) x Chebyshev ShenNeumann 257 with
    alpha = k^2 + 1000 (the headline's shift; the Neumann branch of the
    Helmholtz kernels) in both forms, and ShenDirichlet with wall values
    u(-1) = 1, u(1) = -1 in the mixed form (the boundary-function backward
    and the Helmholtz boundary matrices): scalar product -> solve -> backward
    of a random RHS (seed 0), L2 flushed before every step."""
    import shenfun_gb300 as sg
    f = np.random.default_rng(0).standard_normal((NX, NY, NZ))
    out = {"workload": f"Fourier {NX} (C2C) x Fourier {NY} (R2C) x Chebyshev {NZ}, alpha = k^2 + 1000, "
                       "RHS N(0,1) seed 0", "solve_factors": "FP64 (both forms, as the headline)"}
    cases = (("neumann_plain", {"left": {"N": 0}, "right": {"N": 0}}, "plain"),
             ("neumann_mixed", {"left": {"N": 0}, "right": {"N": 0}}, "mixed"),
             ("dirichlet_walls_mixed", (1.0, -1.0), "mixed"))
    ref = None
    for name, bc, form in cases:
        T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"), sg.FunctionSpace(NY, "F", dtype="d"),
                                         sg.FunctionSpace(NZ, "C", bc=bc)), form=form)
        u, v = sg.TrialFunction(T), sg.TestFunction(T)
        H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + C_SHIFT * u), form="plain")
        fj = sg.Array(T, buffer=f)
        f_hat, u_hat, uq = sg.Function(T), sg.Function(T), sg.Array(T)

        def step():
            sg.inner(v, fj, output_array=f_hat)
            H(f_hat, u_hat)
            T.backward(u_hat.v, uq.v)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ms = float(np.mean(time_steps_gpu(torch, step, steps, flush, st)))
        res = {"ms_per_step": ms, "solves_per_s": 1e3 / ms}
        if name == "neumann_plain":
            ref = uq.v.clone()
        elif name == "neumann_mixed":
            res["rel_err_vs_plain"] = float(((uq.v - ref).abs().max() / ref.abs().max()).item())
        out[name] = res
        del T, H, fj, f_hat, u_hat, uq
    return out


def dealias_leg(torch, flush, st, steps=10):
    """The 3/2-rule dealiased nonlinear term on the channel grid: padded
    backward (Fourier axes 256 -> 384, sgpu_fourier_pad + length-384
    transforms), pointwise square, padded forward (length-384 transforms +
    sgpu_fourier_truncate), Chebyshev ShenDirichlet 257 unpadded, both forms,
    L2 flushed before every step."""
    import shenfun_gb300 as sg
    out = {"workload": f"u_hat -> u^2 (3/2 rule) on Fourier {NX} x Fourier {NY} x Chebyshev {NZ}, "
                       "padded grid 384 x 384 x 257"}
    rng = np.random.default_rng(0)
    shape = (NX, NY // 2 + 1, NZ)
    u0 = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    u0[:, :, NZ - 2:] = 0
    ref = None
    for form in ("plain", "mixed"):
        T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"), sg.FunctionSpace(NY, "F", dtype="d"),
                                         sg.FunctionSpace(NZ, "C", bc=(0, 0))), form=form)
        TP = T.get_dealiased((1.5, 1.5, 1))
        uh = sg.Function(T)
        uh.v.copy_(u0)
        up = sg.Array(TP)
        wh = sg.Function(T)

        def step():
            TP.backward(uh.v, up.v)
            up.v.mul_(up.v)
            TP.forward(up.v, wh.v)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ms = float(np.mean(time_steps_gpu(torch, step, steps, flush, st)))
        res = {"ms_per_step": ms}
        if ref is None:
            ref = wh.v.clone()
        else:
            res["rel_err_vs_plain"] = float(((wh.v - ref).abs().max() / ref.abs().max()).item())
        out[form] = res
        del T, TP, uh, up, wh
    return out


def latency_leg(torch, reps=200):
    """2D Poisson on Fourier 64 (x, [0, 2 pi)) x Chebyshev ShenDirichlet 64
    (y): manufactured u = sin(2x) (1 - y^2) cos(pi y / 2), f = -lap u on the
    quadrature grid; per-solve latency of the round trip (33 systems), eager
    and as one CUDA-graph replay (inputs resident, no L2 flush: a latency
    figure), the error against u, and the reference's CPU path on the same
    grid."""
    import shenfun_gb300 as sg
    Nx = Ny = 64
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="d"), sg.FunctionSpace(Ny, "C", bc=(0, 0))),
                              axes=(1, 0))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u))))
    x = 2 * np.pi * np.arange(Nx) / Nx
    y = np.cos(np.pi * (2 * np.arange(Ny) + 1) / (2 * Ny))
    X, Y = np.meshgrid(x, y, indexing="ij")
    cy, sy = np.cos(np.pi * Y / 2), np.sin(np.pi * Y / 2)
    g = (1 - Y ** 2) * cy
    gpp = -2 * cy + 2 * np.pi * Y * sy - (np.pi ** 2 / 4) * (1 - Y ** 2) * cy
    u_exact = np.sin(2 * X) * g
    f = np.sin(2 * X) * (4 * g - gpp)
    fj = sg.Array(T, buffer=f)
    f_hat, u_hat, uq = sg.Function(T), sg.Function(T), sg.Array(T)

    def step():
        sg.inner(v, fj, output_array=f_hat)
        H(f_hat, u_hat)
        T.backward(u_hat.v, uq.v)

    out = {"workload": "2D Poisson, Fourier 64 x Chebyshev ShenDirichlet 64, u = sin(2x)(1-y^2)cos(pi y/2)"}
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            step()
    torch.cuda.current_stream().wait_stream(s)
    g_ = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_):
        step()
    st = torch.cuda.current_stream()
    for mode, fn in (("eager", step), ("graph", g_.replay)):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        e1.synchronize()
        out[f"us_per_solve_{mode}"] = 1e3 * e0.elapsed_time(e1) / reps
    got = uq.v.cpu().numpy()
    out["rel_err_vs_exact"] = float(np.abs(got - u_exact).max() / np.abs(u_exact).max())
    from oracle.cpu_baseline import Poisson2D, time_calls
    pz = Poisson2D(Nx, Ny)
    ts = time_calls(lambda: pz.step(f), 50, 3)
    out["cpu_baseline"] = {"us_per_solve": 1e6 * float(np.median(ts)), "cores": 1, "kind": pz.kind,
                           "sample": "50 round trips on 1 host thread (scipy.fft for FFTW, reference "
                                     "LU_Helmholtz/Solve_Helmholtz), median",
                           "rel_err_vs_exact": float(np.abs(pz.step(f) - u_exact).max() / np.abs(u_exact).max())}
    return out


def imex_leg(torch, steps=10):
    """IMEX time stepping on the channel grid (the caller of the path,
    utilities/integrators.py:702-900): IMEXRK443 for u_t = nu lap(u) + u^2,
    nu = 1e-3, dt = 1e-3, mixed form; the nonlinear term through the
    transforms (backward, square, scalar product) at every stage, then the
    stage's Helmholtz solve.  Per step: eager launches vs one CUDA-graph
    replay."""
    import shenfun_gb300 as sg
    from shenfun_gb300 import integrators as I
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"), sg.FunctionSpace(NY, "F", dtype="d"),
                                     sg.FunctionSpace(NZ, "C", bc=(0, 0))), form="mixed")
    v = sg.TestFunction(T)
    work = sg.Array(T)

    def N(u_hat, out):
        T.backward(u_hat.v, work.v)
        work.v.mul_(work.v)
        T.scalar_product(work.v, out)

    a = sg.Array(T)
    a.v.copy_(0.1 * torch.randn(a.shape, dtype=torch.float64, device="cuda"))
    u_hat = a.forward()
    sol = I.IMEXRK443(v, u_hat, lambda u: 1e-3 * sg.div(sg.grad(u)), N, 1e-3)
    sol.assemble()
    st = torch.cuda.current_stream()
    out = {"scheme": "IMEXRK443", "stages": 4, "workload": "channel grid, mixed form, N = u^2"}
    for mode in ("eager", "graph"):
        if mode == "graph":
            sol.capture_step(warmup=2)
            fn = sol.replay
        else:
            fn = sol.step
            fn()
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            fn()
        e1.record(st)
        e1.synchronize()
        out[f"ms_per_step_{mode}"] = e0.elapsed_time(e1) / steps
    out["finite"] = bool(torch.isfinite(u_hat.v).all().item())
    return out


CASES = {
    # one transform of the channel grid, for profiler captures:  name -> (kind, form)
    "r2c-plain": ("r2c", "plain"), "r2c-mixed": ("r2c", "mixed"),
    "c2r-mixed": ("c2r", "mixed"), "c2c-plain": ("c2c", "plain"), "c2c-mixed": ("c2c", "mixed"),
    # the mixed form's length-256 passes in 64-bit fixed point (plan variant 5)
    "c2c-fixed": ("c2c", "fixed"), "r2c-fixed": ("r2c", "fixed"), "c2r-fixed": ("c2r", "fixed"),
    # the same C2C with each CTA's input tile staged by a tensor copy (variant 7)
    "c2c-tma": ("c2c", "tma"),
    "bih-plain": ("bih", "plain"), "pad-mixed": ("pad", "mixed"), "bc-mixed": ("bc", "mixed"),
    "cheb-plain": ("cheb", "plain"), "cheb-mixed": ("cheb", "mixed"),
    "solve-plain": ("solve", "plain"),
    # the FP32 sweeps + FP64 residual refinement of the same systems
    "solve-refined": ("solve", "mixed-refined"),
    # one serving batch: 8 problems of Fourier 64 x Fourier 64 x Chebyshev 65
    # (different shifts) through a BatchRunner, eager launches
    "batch-mixed": ("batch", "mixed"),
    "leg-plain": ("leg", "plain"), "leg-mixed": ("leg", "mixed"),
    "leg128-mixed": ("leg128", "mixed"),
    # the whole round-trip step (scalar product, solve, backward)
    "step-plain": ("step", "plain"), "step-mixed": ("step", "mixed"),
    # the 2D Poisson round trip on Fourier 64 x Chebyshev ShenDirichlet 64
    "poisson2d-plain": ("poisson2d", "plain"),
}


def run_case(name, reps=3):
    """Run one kernel of the workload `reps` times (for ncu); prints 'ok'."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from shenfun_gb300 import _lib
    from shenfun_gb300.spaces import R2C, ChebyshevShenDirichlet
    kind, form = CASES[name]
    fixed = form in ("fixed", "tma")
    variant = 7 if form == "tma" else 5
    if fixed:
        form = "mixed"
    x = torch.randn(NX, NY, NZ, dtype=torch.float64, device="cuda")
    if kind in ("r2c", "c2r", "c2c") and fixed:
        from shenfun_gb300.plans import LinePlan
        xk = {"r2c": _lib.XF_R2C, "c2r": _lib.XF_C2R, "c2c": _lib.XF_C2C_FWD}[kind]
        P = LinePlan(xk, 256, form=_lib.MIXED_DF)
        P.variant = variant
        c = torch.randn(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        y = torch.empty_like(c)
        if kind == "r2c":
            fn = lambda: P(x, y, 1, 1.0 / NY)  # noqa: E731
        elif kind == "c2r":
            fn = lambda: P(c, x, 1, 1.0)  # noqa: E731
        else:
            fn = lambda: P(c, y, 0, 1.0 / NX)  # noqa: E731
    elif kind == "r2c":
        V = R2C(NY)
        V.form = _lib.FORMS[form]
        y = torch.empty(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        fn = lambda: V.forward(x, y, axis=1)  # noqa: E731
    elif kind == "c2r":
        V = R2C(NY)
        V.form = _lib.FORMS[form]
        c = torch.randn(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        fn = lambda: V.backward(c, x, axis=1)  # noqa: E731
    elif kind == "c2c":
        from shenfun_gb300.spaces import C2C
        V = C2C(NX)
        V.form = _lib.FORMS[form]
        c = torch.randn(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        y = torch.empty_like(c)
        fn = lambda: V.forward(c, y, axis=0)  # noqa: E731
    elif kind == "bih":
        # biharmonic solve of Fourier 128 x Fourier 128 x ShenBiharmonic 129
        import shenfun_gb300 as sg
        T = sg.TensorProductSpace(sg.comm, (sg.FunctionSpace(128, "F", dtype="D"),
                                            sg.FunctionSpace(128, "F", dtype="d"),
                                            sg.FunctionSpace(129, "C", bc=(0, 0, 0, 0))), form=form)
        u, v = sg.TrialFunction(T), sg.TestFunction(T)
        H = sg.chebyshev.la.Biharmonic(sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u))))))
        b = sg.Function(T, buffer=np.random.default_rng(0).standard_normal(T.shape(True)))
        uh = sg.Function(T)
        fn = lambda: H(b, uh)  # noqa: E731
    elif kind == "pad":
        # 3/2-rule padded backward of the x axis: 256 -> 384 coefficients
        import shenfun_gb300 as sg
        F = sg.FunctionSpace(NX, "F", dtype="D").get_dealiased(1.5)
        F.form = _lib.FORMS[form]
        c = torch.randn(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        y = torch.empty(3 * NX // 2, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        fn = lambda: F.backward(c, y, axis=0)  # noqa: E731
    elif kind == "bc":
        # the forward transform of a Chebyshev axis with wall values 1, -1
        import shenfun_gb300 as sg
        V = sg.FunctionSpace(NZ, "C", bc=(1.0, -1.0))
        V.form = _lib.FORMS[form]
        y = torch.empty_like(x)
        fn = lambda: V.forward(x, y, axis=2)  # noqa: E731
    elif kind == "cheb":
        V = ChebyshevShenDirichlet(NZ)
        V.form = _lib.FORMS[form]
        y = torch.empty_like(x)
        fn = lambda: V.scalar_product(x, y, axis=2)  # noqa: E731
    elif kind == "leg":
        # Legendre ShenDirichlet N = 512 backward over 16,384 lines
        from shenfun_gb300.legendre import LegendreShenDirichlet
        V = LegendreShenDirichlet(512, form=form)
        c = torch.randn(16384, 512, dtype=torch.float64, device="cuda")
        y = torch.empty_like(c)
        fn = lambda: V.backward(c, y, axis=1)  # noqa: E731
    elif kind == "leg128":
        # Legendre ShenDirichlet N = 128 backward over 65,536 lines
        from shenfun_gb300.legendre import LegendreShenDirichlet
        V = LegendreShenDirichlet(128, form=form)
        c = torch.randn(65536, 128, dtype=torch.float64, device="cuda")
        y = torch.empty_like(c)
        fn = lambda: V.backward(c, y, axis=1)  # noqa: E731
    elif kind == "step":
        import shenfun_gb300 as sg
        run = FormRun(sg, form, x.cpu().numpy())
        fn = run.step
    elif kind == "batch":
        from shenfun_gb300.problem import HelmholtzProblem, BatchRunner
        probs = [HelmholtzProblem((64, 64, 65), "chebyshev", c, form) for c in (0.5, 3.0, 10.0, 30.0, 100.0,
                                                                                 300.0, 1e3, 1e4)]
        s = torch.cuda.current_stream()
        br = BatchRunner(probs[0], 8, s, graph=False)
        br.f.copy_(torch.randn(br.f.shape, dtype=torch.float64, device="cuda"))
        fn = lambda: br.run(probs)  # noqa: E731
    elif kind == "poisson2d":
        import shenfun_gb300 as sg
        T = sg.TensorProductSpace(None, (sg.FunctionSpace(64, "F", dtype="d"),
                                         sg.FunctionSpace(64, "C", bc=(0, 0))), axes=(1, 0))
        u, v = sg.TrialFunction(T), sg.TestFunction(T)
        H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u))))
        fj = sg.Array(T, buffer=np.random.default_rng(0).standard_normal((64, 64)))
        f_hat, u_hat, uq = sg.Function(T), sg.Function(T), sg.Array(T)

        def fn():
            sg.inner(v, fj, output_array=f_hat)
            H(f_hat, u_hat)
            T.backward(u_hat.v, uq.v)
    else:
        import shenfun_gb300 as sg
        run = FormRun(sg, form, x.cpu().numpy())
        b = torch.randn(NX, NY // 2 + 1, NZ, dtype=torch.complex128, device="cuda")
        fn = lambda: run.H(b, run.u_hat)  # noqa: E731
    for _ in range(reps):
        fn()
    torch.cuda.synchronize()
    print("ok", name)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the serving and Legendre legs")
    ap.add_argument("--case", choices=sorted(CASES), help="run one kernel case (for profilers)")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case)
    if args.impl == "reference":
        return run_reference(args)
    args.warmup = max(args.warmup, 3)

    import torch
    import __graft_entry__
    __graft_entry__.build()
    import shenfun_gb300 as sg

    ws, rank, local = setup_dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    dev = torch.device("cuda", local)
    st = torch.cuda.current_stream()
    f_np = np.random.default_rng(0).standard_normal((NX, NY, NZ))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    runs = {"plain": FormRun(sg, "plain", f_np), "mixed": FormRun(sg, "mixed", f_np),
            "mixed-refined": FormRun(sg, "mixed-refined", f_np)}

    # reference answer for the error check (outside every timed region)
    ref = None
    if rank == 0:
        from oracle import problems as P
        bases = [("fourier", "C2C", NX), ("fourier", "R2C", NY), ("chebyshev", "SD", NZ)]
        ref, _, _ = P.helmholtz_roundtrip(f_np, bases, C_SHIFT, 2)

    results = {}
    with ClockSampler(local) as clk:
        for name, run in runs.items():
            for _ in range(args.warmup):
                run.step()
            barrier()
            ts_ms = time_steps_gpu(torch, run.step, args.steps, flush, st)
            tot_ms = replica_total_ms(float(ts_ms.sum()), dist, dev)
            err = None
            if ref is not None:
                got = run.uq.v.cpu().numpy()
                err = float(np.abs(got - ref).max() / np.abs(ref).max())
            results[name] = {"value": ws * args.steps / (tot_ms / 1e3), "ms_per_step": tot_ms / args.steps,
                             "p50_ms": float(np.percentile(ts_ms, 50)),
                             "p99_ms": float(np.percentile(ts_ms, 99)),
                             "rel_err_vs_oracle": err,
                             "achieved_roundtrip_GBs": ROUNDTRIP_BYTES / (tot_ms / args.steps / 1e3) / 1e9}
    # the chosen form: the fastest of the mixed forms within the bound
    # against the FP64 oracle (plain when none is)
    ok_forms = [k for k in ("mixed", "mixed-refined") if results[k]["rel_err_vs_oracle"] is not None and
                results[k]["rel_err_vs_oracle"] <= MIXED_TOL]
    chosen = agree(max(ok_forms, key=lambda k: results[k]["value"]) if ok_forms else "plain", dist)
    run = runs[chosen]
    for name in runs:
        results[name]["stage_ms"] = stage_times(torch, runs[name], flush, st)
    stage_ms = results[chosen]["stage_ms"]
    dom = max(stage_ms, key=stage_ms.get)
    # the roofline of every stage is HBM: algorithmic bytes (read + write of
    # the arrays, the factor cache for the solve) over the stage time against
    # the measured copy bandwidth.  The tensor-core passes also report the
    # tensor pipe's share (digit-product flops over the BF16 peak) separately.
    peak, peak_kind = peaks()
    achieved = STAGE_BYTES[dom] / (stage_ms[dom] / 1e3) / 1e9
    roof = {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes": STAGE_BYTES[dom]}
    tensor_util = None
    if chosen != "plain" and dom in TC_STAGES:
        tpeak, tpeak_kind = peaks("bf16_tflops", 1900.0)
        tach = TC_FLOPS / (stage_ms[dom] / 1e3) / 1e12
        tensor_util = {"achieved_tflops": tach, "peak_tflops": tpeak, "frac": tach / tpeak,
                       "peak_source": tpeak_kind, "flops": TC_FLOPS,
                       "note": "28 BF16 digit products per FP64 multiply-add; stage time includes the "
                               "line-scale kernel"}
    tkey = ("mixed" if chosen != "plain" else "plain") + ":" + dom
    traffic = profiled_traffic(tkey)
    if traffic is None and tkey == "mixed:z_backward":
        traffic = profiled_traffic("mixed:z_scalar_product")  # the same kernels, one K step fewer
    stage_frac = {k: STAGE_BYTES[k] / (v / 1e3) / 1e9 / peak for k, v in stage_ms.items()}

    # end to end through the public API with host buffers (pinned), per step:
    # H2D of the RHS, round trip, D2H of the solution
    f_host = torch.from_numpy(f_np).pin_memory()
    u_host = torch.empty((NX, NY, NZ), dtype=torch.float64).pin_memory()
    e2e_steps = max(3, args.steps)

    def e2e_step():
        run.fj.v.copy_(f_host, non_blocking=True)
        run.step()
        u_host.copy_(run.uq.v, non_blocking=True)

    e2e_step()
    barrier()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(e2e_steps):
        e2e_step()
    b.record(st)
    b.synchronize()
    e2e_serial = ws * e2e_steps / (a.elapsed_time(b) / 1e3)
    e2e_val = e2e_pipelined(torch, sg, run, chosen, f_np, f_host, e2e_steps, st) * ws

    serving = legendre = imex = biharmonic = latency = neumann = dealias = refinement = None
    if rank == 0 and not args.no_extra:
        serving = serving_leg(torch)
        legendre = {"sweep": legendre_sweep(torch, flush, st),
                    # beyond one exact K chunk (1024): two chunk launches per contraction
                    "N2048": legendre_leg(torch, flush, st, N=2048, lines=4096, reps=3),
                    # the dense contraction against the DLT's DCT/DST passes alone
                    "dlt_bound": dlt_bound_leg(torch, flush, st)}
        imex = imex_leg(torch)
        biharmonic = biharmonic_leg(torch, flush, st)
        refinement = refinement_leg(torch, flush, st, f_np)
        latency = latency_leg(torch)
        neumann = neumann_leg(torch, flush, st)
        dealias = dealias_leg(torch, flush, st)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rt, ts = cpu_leg(2, 1, 1)
        solver = "reference Cython la.pyx" if rt.kind == "reference" else "numpy port"
        cpu = {"value": len(ts) / float(sum(ts)), "unit": "solves/s", "cores": 1, "kind": rt.kind,
               "sample": f"{len(ts)} full {NX}x{NY}x{NZ} round trips on 1 host thread "
                         f"(scipy.fft for FFTW, {solver} solve), factorisation excluded"}

    if rank == 0:
        r = results[chosen]
        out = {
            "metric": METRIC, "value": r["value"], "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": chosen, "systems": NX * (NY // 2 + 1),
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "latency_ms": {"p50": r["p50_ms"], "p99": r["p99_ms"]},
            "rel_err_vs_oracle": r["rel_err_vs_oracle"],
            "forms": results,
            "chosen_over_plain": results[chosen]["value"] / results["plain"]["value"],
            "roofline": dict(roof, kernel=f"{chosen}:{dom}", achieved=achieved, peak=peak,
                             frac=achieved / peak, traffic=traffic, peak_source=peak_kind,
                             traffic_unit="bytes per stage (ncu, committed profile)" if traffic else None,
                             tensor_util=tensor_util, stage_hbm_frac=stage_frac),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "solves/s",
                    "h2d_bytes_per_step": R_BYTES, "d2h_bytes_per_step": R_BYTES,
                    "mode": "three requests in flight: H2D and D2H on their own streams overlap the "
                            "other requests' round trips",
                    "sequential_value": e2e_serial},
            "gpu_launches": sum(runs[k].launches_per_step for k in runs) * args.steps,
            "clocks": clk.summary(),
            "serving": serving,
            "legendre": legendre,
            "imex": imex,
            "biharmonic": biharmonic,
            "banded_refinement": refinement,
            "small_2d_latency": latency,
            "boundary_conditions": neumann,
            "dealias": dealias,
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
