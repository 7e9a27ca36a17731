#!/usr/bin/env python3
"""Operator-apply throughput of the fused FP64 SIPG-SEM matvec on GB300.

Workload: the 1024 x 1024-element, degree-4 mesh of the unit square (26,214,400
DoF), penalty p^2, input u ~ U[-1, 1] i.i.d. (numpy PCG64, seed 0).  One step
is 100 applies y = A u, the reference's own timing loop
(performance_tests/mvm_performance_test.cu:44-65); the metric is GDoF/s per
apply.  Input and output (209.7 MB each) are larger than the 126 MB L2, so no
flush is needed between applies.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU restatement of the reference's matvec
(oracle/, all host threads) on the same workload, one apply per step.  With N
GPUs (torchrun) every rank runs the same workload on its own GPU (replicas; the
path is one GPU's), `value` is the sum over ranks, the time the max.
Prints one JSON line on rank 0.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cuda-sipg-matrix-free_gb300")
for _p in (PKG, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

DIM, DEGREE = 1024, 4
PEN = float(DEGREE * DEGREE)
NDOF = DIM * DIM * (DEGREE + 1) ** 2
APPLIES_PER_STEP = 100
BYTES_PER_DOF = 16  # read u once, write y once (FP64)
# FP64-pipe operations per DoF issued by the fused FP64 kernel (column form),
# counted as two flops each: one chain per output of 2n + 4 (face corrections
# as its seed, weighted volume sums, the four liftings), face derivatives 4,
# face combines 12/n, corner additions 4/n^2
FP64_FLOPS_PER_DOF = 2.0 * (2 * (DEGREE + 1) + 8 + 12.0 / (DEGREE + 1) + 4.0 / (DEGREE + 1) ** 2)
THESIS_K20X_GDOFS = 1.031  # Thesis_TEXT.pdf p.54 T4.15: 1024^2, p=4, volume+flux on a K20X
METRIC = "GDoF/s per SIPG apply (FP64, 1024x1024 elements, p=4)"
CONFIG = {
    "workload": "fused SIPG-SEM apply y = A u, 1024x1024 quads, p=4, pen=16, 100 applies per step",
    "dim": DIM, "degree": DEGREE, "pen": PEN, "ndof": NDOF, "applies_per_step": APPLIES_PER_STEP,
    "l2": "no flush: input and output are 209.7 MB each, larger than the 126 MB L2",
}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def copy_bound_ms(torch, h_in, h_out, reps=10):
    """ms to move one step's input host->device and output device->host at
    once (two streams, pinned buffers): the floor of an end-to-end step."""
    d_a = torch.empty(h_in.numel(), dtype=h_in.dtype, device="cuda")
    d_b = torch.empty(h_out.numel(), dtype=h_out.dtype, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def both():
        with torch.cuda.stream(s1):
            d_a.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(s2):
            h_out.copy_(d_b, non_blocking=True)

    both()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        both()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps * 1e3


def traffic_per_launch():
    """DRAM bytes per apply launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "apply_f64_1024_p4_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest of `value` over the ranks of the process group (a timing:
    the slowest rank's), or `value` itself in a single process."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, units_per_step, ms):
    """Whole-job units per second of `world` replicas that each processed
    steps x units_per_step in the slowest replica's `ms` milliseconds."""
    return world * steps * units_per_step / (ms * 1e-3)


def cpu_apply_rate(seconds=10.0, max_reps=20):
    """The oracle (CPU restatement of the reference matvec) on all host threads."""
    import numpy as np

    import oracle_lib

    orc = oracle_lib.load()
    nthreads = os.cpu_count() or 1
    x = np.random.default_rng(0).uniform(-1.0, 1.0, NDOF)
    orc.apply(DEGREE, DIM, PEN, x, nthreads=nthreads)  # warm-up
    reps, t0 = 0, time.perf_counter()
    while reps < max_reps and (reps == 0 or time.perf_counter() - t0 < seconds):
        orc.apply(DEGREE, DIM, PEN, x, nthreads=nthreads)
        reps += 1
    dt = time.perf_counter() - t0
    return {"value": reps * NDOF / dt / 1e9, "unit": "GDoF/s", "cores": nthreads, "kind": "port",
            "sample": "%d full applies of the 1024x1024 p=4 workload (%.1f s)" % (reps, dt)}


def reference_kernels_same_gpu(x, y, reps=20):
    """The reference's own volume + flux_term6a + flux_term6b, compiled for sm_103a
    from its headers (oracle/_ref/ref_kernels.cubin), timed on this GPU."""
    import oracle_lib

    if not oracle_lib.ref_gpu_available():
        return None
    ms = oracle_lib.ref_gpu().apply(DEGREE, DIM, PEN, x.data_ptr(), y.data_ptr(), reps)
    return {"value": reps * NDOF / (ms * 1e-3) / 1e9, "unit": "GDoF/s", "applies": reps,
            "source": "reference kernels (volume, flux_term6a, flux_term6b) built unchanged for sm_103a, "
                      "launched with the reference geometry, CUDA events"}


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import numpy as np

    import oracle_lib

    orc = oracle_lib.load()
    nthreads = os.cpu_count() or 1
    x = np.random.default_rng(0).uniform(-1.0, 1.0, NDOF)
    for _ in range(args.warmup):
        orc.apply(DEGREE, DIM, PEN, x, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.apply(DEGREE, DIM, PEN, x, nthreads=nthreads)
    dt = time.perf_counter() - t0
    value = args.steps * NDOF / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / THESIS_K20X_GDOFS, "dtype": "f64",
        "data": "synthetic: u ~ U[-1,1] i.i.d., numpy PCG64 seed 0",
        "config": dict(CONFIG, applies_per_step=1,
                       reference="CPU restatement of the reference matvec (oracle/sipg_oracle.c), bit-exact with "
                                 "the reference's volume + flux_term6a + flux_term6b; the reference has no CPU path"),
        "cpu_baseline": {"value": value, "unit": "GDoF/s", "cores": nthreads, "kind": "port",
                         "sample": "%d full applies of the 1024x1024 p=4 workload" % args.steps},
        "e2e": {"value": value, "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import sipg_gb300 as sipg

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        pg = dist
    op = sipg.Operator(DIM, DEGREE, PEN)
    x_np = np.random.default_rng(0).uniform(-1.0, 1.0, NDOF)
    x = torch.from_numpy(x_np).cuda()
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        for _ in range(APPLIES_PER_STEP):
            op.apply(x, y)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.25)
    n0 = sipg.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        for _ in range(APPLIES_PER_STEP):
            op.apply(x, y)
    e1.record(stream)
    e1.synchronize()
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), pg, "cuda")
    if pg:
        pg.barrier()
    ms_per_step = ms / args.steps
    value = replica_throughput(world, args.steps, APPLIES_PER_STEP * NDOF, ms) / 1e9

    # end to end through the public C ABI with pinned host buffers: every step
    # copies the input to the device, applies once, copies the result back
    h_in = torch.from_numpy(x_np).pin_memory()
    h_out = torch.empty(NDOF, dtype=torch.float64).pin_memory()
    e2e_steps = max(3, min(args.steps, 20))
    L = sipg.lib()
    import ctypes as C

    def host_apply():
        st = L.sipg_apply_host_f64(op._h, C.c_void_p(h_in.data_ptr()), C.c_void_p(h_out.data_ptr()),
                                   C.c_void_p(stream.cuda_stream))
        if st != 0:
            raise sipg.SipgError(st, L.sipg_last_error().decode())

    host_apply()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_apply()
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg, "cuda")
    e2e_value = replica_throughput(world, e2e_steps, NDOF, e2e_s * 1e3) / 1e9
    ok = bool(np.array_equal(h_out.numpy(), y.cpu().numpy()))
    copy_ms = copy_bound_ms(torch, h_in, h_out)

    peak, peak_src = measured_peaks()
    dur = ms * 1e-3 / (args.steps * APPLIES_PER_STEP)
    achieved = BYTES_PER_DOF * NDOF / dur / 1e9
    fp64_peak, fp32_peak = sipg.probe_fma_peak()
    fp64_achieved = FP64_FLOPS_PER_DOF * NDOF / dur / 1e12
    traffic = traffic_per_launch()
    line = {
        "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / THESIS_K20X_GDOFS, "dtype": "f64",
        "data": "synthetic: u ~ U[-1,1] i.i.d., numpy PCG64 seed 0",
        "config": dict(CONFIG, parallelism="replicas" if world > 1 else "single GPU"),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "GDoF/s", "h2d_bytes_per_step": NDOF * 8, "d2h_bytes_per_step": NDOF * 8,
                "steps": e2e_steps, "api": "sipg_apply_host_f64 (pinned host buffers, one apply per step)",
                "matches_device_result": ok,
                "copy_bound": {"ms_per_step": copy_ms, "gdofs": NDOF / (copy_ms * 1e-3) / 1e9,
                               "what": "the step's H2D and D2H run at once on two streams (torch copies), no apply"}},
        "gpu_launches": launches,
        "roofline": {
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_src,
            "algorithmic_bytes_per_dof": BYTES_PER_DOF, "launch_ms": dur * 1e3,
            "fp64_pipe": {"achieved_tflops": fp64_achieved, "peak_tflops": fp64_peak, "frac": fp64_achieved / fp64_peak,
                          "flops_per_dof": FP64_FLOPS_PER_DOF,
                          "peak_source": "measured live (sipg_probe_fma_peak, independent DFMA chains)"},
        },
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_apply_rate()
        try:
            line["reference_kernels_same_gpu"] = reference_kernels_same_gpu(x, y)
        except Exception as exc:  # the baseline is optional; the product line stands
            line["reference_kernels_same_gpu"] = {"unavailable": str(exc)}
    op.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# The other benchmark configurations (parity-test cases of the headline path
# and the solver additions), one JSON line each: --config sweep | solve16 |
# mixed | batch | serve.  Each keeps the timing rules: warm-up first, CUDA
# events or a synchronised wall clock, clocks sampled during the timed part.
# ---------------------------------------------------------------------------


def _base_line(args, metric, value, unit, higher, dtype, config, **extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic (seeded)", "config": config}
    line.update(extra)
    return line


def _timed(torch, fn, steps):
    """ms per call of fn() over `steps` calls, CUDA events on the current stream."""
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        fn()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def run_sweep(args):
    """Apply throughput at ~16M DoF for p = 1..8, N = round(4000 / (p + 1))."""
    import numpy as np
    import torch

    import sipg_gb300 as sipg

    rows = {}
    tot_dof = tot_ms = 0.0
    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    for p in range(1, 9):
        d = round(4000 / (p + 1))
        op = sipg.Operator(d, p, float(p * p))
        x = torch.from_numpy(np.random.default_rng(0).uniform(-1.0, 1.0, op.ndof)).cuda()
        y = torch.empty_like(x)
        for _ in range(args.warmup):
            op.apply(x, y)
        ms = _timed(torch, lambda: op.apply(x, y), max(args.steps, 10))
        row = {"dim": d, "ndof": op.ndof, "gdofs": op.ndof / ms / 1e6, "gbs": 16 * op.ndof / ms / 1e6}
        try:
            import oracle_lib

            if oracle_lib.ref_gpu_available():
                reps = 5
                rms = oracle_lib.ref_gpu().apply(p, d, float(p * p), x.data_ptr(), y.data_ptr(), reps) / reps
                row["reference_kernels_gdofs"] = op.ndof / rms / 1e6
                row["speedup_vs_reference_kernels"] = rms / ms
        except Exception as exc:
            row["reference_kernels"] = "unavailable: %s" % exc
        rows["p%d" % p] = row
        tot_dof += op.ndof
        tot_ms += ms
        op.close()
    clocks = sampler.stop()
    value = tot_dof / tot_ms / 1e6
    line = _base_line(args, "GDoF/s per SIPG apply, ~16M DoF, p = 1..8 (aggregate: total DoF / total time)", value,
                      "GDoF/s", True, "f64",
                      {"workload": "apply sweep: N = round(4000/(p+1)), p = 1..8, pen p^2, u ~ U[-1,1] seed 0",
                       "l2": "inputs 128 MB+ per vector"},
                      per_degree=rows, clocks=clocks, gpu_launches=sipg.launch_count() - n0)
    print(json.dumps(line), flush=True)
    return 0


def run_solve16(args):
    """The 16 x 16, p = 4 solve to relative residual 1e-12 (one solve per step),
    end to end from a host right-hand side to a host solution."""
    import numpy as np
    import torch

    import sipg_gb300 as sipg

    dim, p, pen = 16, 4, 16.0
    op = sipg.Operator(dim, p, pen)
    b_dev = op.rhs("sinsin")
    h_b = b_dev.cpu().pin_memory()
    h_x = torch.empty_like(h_b).pin_memory()
    x = torch.zeros_like(b_dev)
    b = torch.empty_like(b_dev)
    res = {}

    def step():
        b.copy_(h_b, non_blocking=True)
        x.zero_()
        st, r = op.cg(x, b, 1e-12, relative=True)
        h_x.copy_(x, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        res["r"] = r

    for _ in range(args.warmup):
        step()
    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    wall = (time.perf_counter() - t0) / args.steps
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    r = res["r"]
    l2, h1, mx = op.err_norms("sinsin", x)
    extra = {"iterations": r.iterations, "device_ms_per_solve": r.time_ms, "L2": l2, "H1": h1, "max_err": mx,
             "e2e": {"value": 1.0 / wall, "unit": "solves/s", "h2d_bytes_per_step": op.ndof * 8,
                     "d2h_bytes_per_step": op.ndof * 8, "api": "sipg_cg_f64 with host b in, host x out"},
             "ms_per_step": wall * 1e3, "clocks": clocks, "gpu_launches": launches}
    try:
        import oracle_lib

        if oracle_lib.ref_gpu_available():
            xr = torch.zeros_like(b_dev)
            it, ms = oracle_lib.ref_gpu().cg(p, dim, pen, xr.data_ptr(), b_dev.data_ptr(),
                                             1e-12 * float(b_dev.norm().item()))
            extra["reference_kernels_same_gpu"] = {"iterations": it, "ms_per_solve": ms,
                                                   "solves_per_s": 1e3 / ms,
                                                   "source": "reference kernels + its CG loop (cuBLAS dots)"}
    except Exception as exc:
        extra["reference_kernels_same_gpu"] = {"unavailable": str(exc)}
    if not args.no_cpu_baseline:
        import oracle_lib

        orc = oracle_lib.load()
        bn = b_dev.cpu().numpy()
        t0 = time.perf_counter()
        reps = 0
        while reps < 3 or time.perf_counter() - t0 < 2.0:
            it, _, _ = orc.cg(p, dim, pen, bn, 1e-12, rel=True)
            reps += 1
        dt = (time.perf_counter() - t0) / reps
        extra["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                                 "sample": "%d solves, %d iterations each" % (reps, it)}
    # h-convergence over dim = 4..512 (p = 4, same problem, pen p^2, CG to 1e-12
    # relative): error norms and their rates log2(e(h) / e(h/2))
    hs = []
    for dd in (4, 8, 16, 32, 64, 128, 256, 512):
        oph = sipg.Operator(dd, p, pen)
        bh = oph.rhs("sinsin")
        xh = torch.zeros_like(bh)
        sth, rh = oph.cg(xh, bh, 1e-12, relative=True)
        e = oph.err_norms("sinsin", xh)
        hs.append({"dim": dd, "iterations": rh.iterations, "status": sth, "L2": e[0], "H1": e[1], "max": e[2],
                   "ms": rh.time_ms})
        oph.close()
    for a, b2 in zip(hs, hs[1:]):
        b2["rate_L2"] = float(np.log2(a["L2"] / b2["L2"]))
        b2["rate_H1"] = float(np.log2(a["H1"] / b2["H1"]))
    extra["h_convergence_p4"] = hs
    line = _base_line(args, "solves/s, 16x16 quads p=4 SIPG-SEM Poisson CG to relative residual 1e-12",
                      1e3 / r.time_ms, "solves/s", True, "f64",
                      {"workload": "16x16 quads, p=4 (6400 DoF), pen 16, f = 8 pi^2 sin(2 pi x) sin(2 pi y), x0 = 0"},
                      **extra)
    print(json.dumps(line), flush=True)
    op.close()
    return 0


def run_mixed(args):
    """512 x 512, p = 6: mixed-precision solve vs the FP64 CG, both to 1e-10."""
    import torch

    import sipg_gb300 as sipg

    dim, p, pen = 512, 6, 36.0
    op = sipg.Operator(dim, p, pen)
    b = op.rhs("sinsin")
    x64 = torch.zeros_like(b)
    xm = torch.zeros_like(b)
    out = {}

    def fp64():
        x64.zero_()
        out["r64"] = op.cg(x64, b, 1e-10, relative=True)[1]

    def mixed():
        xm.zero_()
        out["st"], out["rm"] = op.solve_mixed(xm, b, 0.1, 1e-10)

    for _ in range(max(1, args.warmup // 3)):
        fp64()
        mixed()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    steps = max(2, min(args.steps, 5))
    ms64 = _timed(torch, fp64, steps)
    msm = _timed(torch, mixed, steps)
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    r64, rm = out["r64"], out["rm"]
    e64 = op.err_norms("sinsin", x64)
    em = op.err_norms("sinsin", xm)
    diff = float(((xm - x64).norm() / x64.norm()).item())
    line = _base_line(args, "solves/s to relative residual 1e-10, 512x512 quads p=6, mixed precision", 1e3 / msm,
                      "solves/s", True, "f32 pairs (inner) + f64 (outer)",
                      {"workload": "512x512 quads, p=6 (12.8M DoF), pen 36, sin-sin f, x0 = 0, rel. residual 1e-10"},
                      ms_per_step=msm, fp64={"solves_per_s": 1e3 / ms64, "iterations": r64.iterations,
                                             "L2": e64[0], "H1": e64[1]},
                      mixed={"status": out["st"], "inner_kind": ["", "f32", "pairs"][rm.inner_kind],
                             "inner_iterations": rm.inner_iterations, "fp64_updates": rm.outer_iterations,
                             "rel_residual": rm.rel_residual, "L2": em[0], "H1": em[1],
                             "rel_diff_vs_fp64_solution": diff},
                      speedup_vs_fp64=ms64 / msm, clocks=clocks, gpu_launches=launches)
    print(json.dumps(line), flush=True)
    op.close()
    return 0


def _batch_case(torch, sipg, workloads, probs):
    """Batched mixed solve of `probs` [(dim, p, pen, modes)] vs one-at-a-time FP64."""
    batch = sipg.Batch([(d, p, pen) for d, p, pen, _ in probs])
    bs = [batch.op(k).rhs("modes", sipg.Modes.make(*m)) for k, (_, _, _, m) in enumerate(probs)]
    xs = [torch.zeros_like(b) for b in bs]

    def solve_batch():
        for x in xs:
            x.zero_()
        return batch.solve_mixed(xs, bs)

    solve_batch()  # warm-up: graph capture
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, res = solve_batch()
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    ok = sum(1 for r in res if r.converged)
    # one at a time, plain FP64 CG (operators reused across equal problems)
    ops = {}
    t_seq = 0.0
    worst = 0.0
    for k, (d, p, pen, _) in enumerate(probs):
        key = (d, p, pen)
        if key not in ops:
            ops[key] = sipg.Operator(d, p, pen)
        x = torch.zeros_like(bs[k])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ops[key].cg(x, bs[k], 1e-10, relative=True)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t0
        worst = max(worst, float(((xs[k] - x).norm() / max(x.norm().item(), 1e-300)).item()))
    for op in ops.values():
        op.close()
    n = len(probs)
    out = {"problems": n, "status": st, "converged": ok, "batch_solves_per_s": n / t_batch,
           "fp64_one_at_a_time_solves_per_s": n / t_seq, "speedup": t_seq / t_batch,
           "max_rel_diff_vs_fp64": worst, "total_dof": sum(workloads.ndof(d, p) for d, p, _, _ in probs),
           "inner_iterations_max": max(r.inner_iterations for r in res)}
    batch.close()
    return out


def run_batch(args):
    import torch

    import sipg_gb300 as sipg
    import workloads

    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    a = _batch_case(torch, sipg, workloads, workloads.shared_mesh_rhs(64, 256, 4, seed=1))
    b = _batch_case(torch, sipg, workloads, workloads.uneven_problems(args.uneven, seed=2))
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    line = _base_line(args, "solves/s, batched mixed-precision solves to 1e-10 (64 RHS on 256x256 p=4)",
                      a["batch_solves_per_s"], "solves/s", True, "f32 pairs (inner) + f64 (outer)",
                      {"workload": "(a) 64 RHS, 256x256 quads p=4, 4 sine modes each (seed 1); "
                                   "(b) %d problems, N log-uniform [16,256], p in 2..8 (seed 2)" % args.uneven},
                      shared_mesh=a, uneven=b, clocks=clocks, gpu_launches=launches)
    print(json.dumps(line), flush=True)
    return 0


def _serve_stream(sipg, reqs, precision, max_active=256):
    srv = sipg.Server(budget_bytes=150 << 30, max_active=max_active, iters_per_step=8)
    pending = list(reqs)
    inflight = {}
    lat, failed = [], 0
    t0 = time.perf_counter()
    i = 0
    while i < len(pending) or inflight:
        now = time.perf_counter() - t0
        while i < len(pending) and pending[i][0] <= now:
            _, d, p, pen, m, tol = pending[i]
            rid, st = srv.submit(d, p, pen, tol, "modes", sipg.Modes.make(*m), precision=precision)
            if st == 0:
                inflight[rid] = i
            else:
                failed += 1
            i += 1
        if not inflight:
            time.sleep(max(0.0, min(0.01, pending[i][0] - now)) if i < len(pending) else 0)
            continue
        srv.step()
        for rid in list(inflight):
            r = srv.poll(rid)
            if r.done:
                if r.status == 0:
                    lat.append(r.latency_ms)
                else:
                    failed += 1
                srv.release(rid)
                del inflight[rid]
    wall = time.perf_counter() - t0
    srv.close()
    lat.sort()
    q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))] if lat else None
    return {"requests": len(reqs), "completed": len(lat), "failed": failed, "wall_s": wall,
            "solves_per_s": len(lat) / wall, "p50_ms": q(0.5), "p99_ms": q(0.99), "max_ms": lat[-1] if lat else None}


def run_serve(args):
    """The request stream at a few arrival rates, mixed-precision requests and
    plain FP64 requests through the same server."""
    import sipg_gb300 as sipg
    import workloads

    rates = [float(r) for r in str(args.rate).split(",")]
    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    sweep = []
    for rate in rates:
        reqs = workloads.request_stream(count=args.requests, rate=rate, seed=3)
        sweep.append({"rate_per_s": rate, "mixed": _serve_stream(sipg, reqs, sipg.F32),
                      "fp64": _serve_stream(sipg, reqs, sipg.F64)})
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    head = sweep[len(sweep) // 2]
    line = _base_line(args, "p99 latency (ms), solve server, mixed precision, at %g requests/s" % head["rate_per_s"],
                      head["mixed"]["p99_ms"], "ms", False, "f32 pairs (inner) + f64 (outer)",
                      {"workload": "%d requests per rate, Poisson arrivals, N log-uniform [8,512], p in 2..8, "
                                   "tol in {1e-8, 1e-10} (seed 3); 150 GB budget" % args.requests},
                      sweep=sweep, clocks=clocks, gpu_launches=launches)
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", choices=("apply", "sweep", "solve16", "mixed", "batch", "serve"), default="apply",
                    help="apply: the headline (1024x1024 p=4 apply); the others are the solver's other workloads")
    ap.add_argument("--uneven", type=int, default=200, help="batch: number of uneven problems")
    ap.add_argument("--requests", type=int, default=100, help="serve: requests per arrival rate")
    ap.add_argument("--rate", default="2,5,10", help="serve: arrival rates per second, comma-separated")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "apply":
        import torch

        torch.cuda.set_device(0)
        return {"sweep": run_sweep, "solve16": run_solve16, "mixed": run_mixed, "batch": run_batch,
                "serve": run_serve}[args.config](args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
