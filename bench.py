"""Benchmark: 3D channel Helmholtz round trips on one GB300.

Workload (the configuration the headline metric is quoted on): Fourier 256
(C2C, x) x Fourier 256 (R2C, y) x Chebyshev ShenDirichlet 257 (z),
alpha = k^2 + 1/(nu dt) with nu dt = 1e-3, RHS i.i.d. N(0, 1) in physical
space from seed 0.  One step = scalar product of the RHS (inner(v, f)) ->
batched Helmholtz solve (33,024 band systems, one per (kx, ky)) -> backward
transform.  The factorisation is set-up work (done once, as in shenfun).

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
METRIC = "Helmholtz solves/s (chosen vs plain FP64, rel err <=1e-10); p50/p99 latency"
WORKLOAD = "3D channel Helmholtz round trip: Fourier 256 (C2C) x Fourier 256 (R2C) x Chebyshev ShenDirichlet 257, alpha=k^2+1/(nu*dt), nu*dt=1e-3, RHS N(0,1) seed 0"

# algorithmic bytes per launch (read + write of each array touched once)
R_BYTES = NX * NY * NZ * 8                      # physical real array
C_BYTES = NX * (NY // 2 + 1) * NZ * 16          # spectral complex array
F_BYTES = NX * (NY // 2 + 1) * NZ * 8           # one factor array
STAGE_BYTES = {
    "z_scalar_product": 2 * R_BYTES,
    "y_r2c": R_BYTES + C_BYTES,
    "x_c2c_fwd": 2 * C_BYTES,
    "helmholtz_solve": 2 * C_BYTES + 4 * F_BYTES,
    "x_c2c_bwd": 2 * C_BYTES,
    "y_c2r": C_BYTES + R_BYTES,
    "z_backward": 2 * R_BYTES,
}


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
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


def setup_dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_leg(steps, warmup, threads, sample_solves=None):
    """Time the reference's CPU path on the full workload (bounded: a few solves)."""
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
                                   f"solve single-threaded ({'reference Cython la.pyx' if rt.kind == 'reference' else 'numpy port'}); "
                                   f"factorisation excluded ({rt.setup_s:.2f} s)"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import __graft_entry__
    __graft_entry__.build()
    import shenfun_gb300 as sg
    from shenfun_gb300 import _lib

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
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(NX, "F", dtype="D"),
                                     sg.FunctionSpace(NY, "F", dtype="d"),
                                     sg.FunctionSpace(NZ, "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + C_SHIFT * u))
    f_np = np.random.default_rng(0).standard_normal((NX, NY, NZ))
    fj = sg.Array(T, buffer=f_np)
    f_hat = sg.Function(T)
    u_hat = sg.Function(T)
    uq = sg.Array(T)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        sg.inner(v, fj, output_array=f_hat)
        H(f_hat, u_hat)
        T.backward(u_hat.v, uq.v)

    launches_per_step = 7
    for _ in range(args.warmup):
        step()
    barrier()
    st = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        for i in range(args.steps):
            flush.zero_()
            evs[i][0].record(st)
            step()
            evs[i][1].record(st)
        barrier()
    ts_ms = np.array([a.elapsed_time(b) for a, b in evs])
    tot_ms = float(ts_ms.sum())
    if dist is not None:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = ws * args.steps / (tot_ms / 1e3)

    # accuracy of the measured path against the oracle (outside the timed region)
    rel_err = None
    if rank == 0:
        from oracle import problems as P
        bases = [("fourier", "C2C", NX), ("fourier", "R2C", NY), ("chebyshev", "SD", NZ)]
        ref, _, _ = P.helmholtz_roundtrip(f_np, bases, C_SHIFT, 2)
        got = uq.v.cpu().numpy()
        rel_err = float(np.abs(got - ref).max() / np.abs(ref).max())

    # per-stage kernel times (CUDA events on the launching stream)
    stage_ms = {}
    spaces = T.bases
    work_r = torch.empty((NX, NY, NZ), dtype=torch.float64, device=dev)
    work_c = torch.empty((NX, NY // 2 + 1, NZ), dtype=torch.complex128, device=dev)
    work_c2 = torch.empty_like(work_c)
    stages = [
        ("z_scalar_product", lambda: spaces[2].scalar_product(fj.v, work_r, axis=2)),
        ("y_r2c", lambda: spaces[1].scalar_product(work_r, work_c, axis=1)),
        ("x_c2c_fwd", lambda: spaces[0].scalar_product(work_c, work_c2, axis=0)),
        ("helmholtz_solve", lambda: H(work_c2, work_c)),
        ("x_c2c_bwd", lambda: spaces[0].backward(work_c, work_c2, axis=0)),
        ("y_c2r", lambda: spaces[1].backward(work_c2, work_r, axis=1)),
        ("z_backward", lambda: spaces[2].backward(work_r, uq.v, axis=2)),
    ]
    reps = 5
    for name, fn in stages:
        fn()
        torch.cuda.synchronize()
        acc = 0.0
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            fn()
            b.record(st)
            b.synchronize()
            acc += a.elapsed_time(b)
        stage_ms[name] = acc / reps
    dom = max(stage_ms, key=stage_ms.get)
    peak, peak_kind = peaks()
    achieved = STAGE_BYTES[dom] / (stage_ms[dom] / 1e3) / 1e9
    traffic = None
    tp = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get(dom)
        except Exception:
            traffic = None

    # end to end through the public API with host buffers (pinned), per step:
    # H2D of the RHS, round trip, D2H of the solution
    f_host = torch.from_numpy(f_np).pin_memory()
    u_host = torch.empty((NX, NY, NZ), dtype=torch.float64).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))

    def e2e_step():
        fj.v.copy_(f_host, non_blocking=True)
        step()
        u_host.copy_(uq.v, non_blocking=True)

    e2e_step()
    barrier()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(e2e_steps):
        e2e_step()
    b.record(st)
    b.synchronize()
    e2e_val = ws * e2e_steps / (a.elapsed_time(b) / 1e3)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rt, ts = cpu_leg(2, 1, 1)
        cpu = {"value": len(ts) / float(sum(ts)), "unit": "solves/s", "cores": 1, "kind": rt.kind,
               "sample": f"{len(ts)} full {NX}x{NY}x{NZ} round trips on 1 host thread "
                         f"(scipy.fft for FFTW, {'reference Cython la.pyx' if rt.kind == 'reference' else 'numpy port'} solve), "
                         "factorisation excluded"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "plain FP64", "systems": NX * (NY // 2 + 1),
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "latency_ms": {"p50": float(np.percentile(ts_ms, 50)),
                           "p99": float(np.percentile(ts_ms, 99))},
            "rel_err_vs_oracle": rel_err,
            "stage_ms": stage_ms,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_kind,
                         "algorithmic_bytes": STAGE_BYTES[dom]},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "solves/s",
                    "h2d_bytes_per_step": R_BYTES, "d2h_bytes_per_step": R_BYTES},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
