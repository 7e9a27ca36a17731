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
# Algorithmic HBM bytes per DoF of the solver steps (each vector a kernel must
# read or write, once):
CG64_BYTES_PER_IT = 80       # FP64 CG iteration: apply (read r, p; write p, Ap) + update (read x, p, r, Ap; write x, r)
FP32_INNER_BYTES_PER_IT = 48  # FP32 inner iteration with the two-level preconditioner: z = M r (read r, write z),
                              # the CG-mode apply (read z, p; write p, Ap), the update (read x, p, r, Ap; write x, r);
                              # the preconditioner's vertex levels (~1 B/DoF) are left out
FLEX_OUTER_BYTES = 120       # flexible outer step: inner restart 16 + gamma 12 + direction 28 + FP64 apply 16 + update 48
RESID_BYTES = 24             # r = b - A x in FP64: read x, b; write r
RELIABLE_UPDATE_BYTES = 64   # reliable update: x += e 24, r = b - A x 24, inner restart 16
MIXED_INNER_TOL = 3e-2       # the flexible solve's inner tolerance (measured fastest at 512^2, p = 6: 54 ms, 1e-2: 56)


def fp64_flops_per_dof(p):
    """FP64 flops per DoF of one fused FP64 apply of degree p (column form)."""
    return 2.0 * (2 * (p + 1) + 8 + 12.0 / (p + 1) + 4.0 / (p + 1) ** 2)
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
    del x, y
    if rank == 0 and world == 1 and not args.no_secondary:
        # the metric's other two parts, measured in the same process: solves/s
        # to a true 1e-10 (mixed vs FP64) and the serving stream's p50 / p99,
        # plus the 16 x 16 solve; each with its own clock record
        import workloads

        cpu = not args.no_cpu_baseline
        for key, fn in (("mixed", lambda: mixed_metrics(torch, sipg, reps=3, cpu=cpu, fp64_peak=fp64_peak)),
                        ("solve16", lambda: solve16_metrics(torch, sipg, steps=20, warmup=3, cpu=cpu)),
                        ("serve", lambda: serve_metrics(sipg, workloads, 50.0, args.serve_requests, cpu=cpu))):
            smp = ClockSampler(local)
            smp.start()
            n1 = sipg.launch_count()
            try:
                line[key] = fn()
            except Exception as exc:  # a secondary part failing must not hide the headline
                line[key] = {"error": "%s: %s" % (type(exc).__name__, exc)}
            line[key]["gpu_launches"] = sipg.launch_count() - n1
            line[key]["clocks"] = smp.stop()
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


def _roofline_solve(bytes_total, ms, fp64_applies, ndof, p, fp64_peak):
    """Time-to-tolerance against the HBM roofline (algorithmic bytes of the
    whole solve / time / measured copy peak) and the FP64-pipe fraction."""
    peak, src = measured_peaks()
    achieved = bytes_total / (ms * 1e-3) / 1e9
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % src, "algorithmic_bytes": bytes_total}
    if fp64_peak:
        fl = fp64_applies * fp64_flops_per_dof(p) * ndof / (ms * 1e-3) / 1e12
        out["fp64_pipe"] = {"achieved_tflops": fl, "peak_tflops": fp64_peak, "frac": fl / fp64_peak,
                            "fp64_applies": fp64_applies}
    return out


def _true_rel(op, x, b):
    """||b - A x|| / ||b||, recomputed in FP64 from the returned solution
    (sipg_residual_f64: the operator's zero-sum contractions over differences,
    whose rounding stays far below the plain sums' on a smooth solution)."""
    return float(op.true_residual(x, b))


def _plain_rel(op, x, b):
    """The same with the plain FP64 apply (sipg_apply_f64), whose rounding puts
    a floor near 1e-10 under it on the larger smooth problems."""
    return float((b - op.apply(x)).norm().item() / b.norm().item())


def _time_solves(torch, fn, reps):
    """(ms per solve, last result): CUDA events on the current stream around
    each call, the median of `reps` after one untimed call."""
    fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    times, res = [], None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        res = fn()
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2], res


def mixed_metrics(torch, sipg, reps=3, cpu=True, fp64_peak=None, dim=512, p=6, inner_tol=MIXED_INNER_TOL):
    """The mixed-precision solve to a TRUE relative residual of 1e-10 (512 x
    512, p = 6, 12.8 M DoF, f = 8 pi^2 sin sin) against the FP64 solvers on the
    same GPU: the reference's CG (stops on its recursive residual; its true
    residual is reported) and FP64 CG with reliable updates (reaches a true
    1e-10).  Every arm states its true residual and its L2 / H1 errors."""
    pen = float(p * p)
    op = sipg.Operator(dim, p, pen)
    b = op.rhs("sinsin")
    n = op.ndof
    x = torch.zeros_like(b)
    arms = {}

    def record(name, ms, iters, fp64_applies, bytes_total, extra):
        l2, h1, mx = op.err_norms("sinsin", x)
        arms[name] = dict({"ms": ms, "solves_per_s": 1e3 / ms, "true_rel_residual": _true_rel(op, x, b),
                           "true_rel_residual_plain_sums": _plain_rel(op, x, b),
                           "L2": l2, "H1": h1, "max_err": mx,
                           "roofline": _roofline_solve(bytes_total, ms, fp64_applies, n, p, fp64_peak)}, **extra)
        if iters is not None:
            arms[name]["iterations"] = iters

    def cg():
        x.zero_()
        return op.cg(x, b, 1e-10, relative=True)

    ms, (st, r) = _time_solves(torch, cg, reps)
    record("fp64_cg", ms, r.iterations, r.iterations, (8 + RESID_BYTES + r.iterations * CG64_BYTES_PER_IT) * n,
           {"status": st, "solver": "the reference's CG (conjugate_gradient_gpu.hpp:18-109), relative 1e-10 on its "
                                    "recursively updated residual"})
    x_ref = x.clone()

    def reliable64():
        x.zero_()
        return op.solve_mixed(x, b, inner_tol=0.1, outer_tol=1e-10, inner="f64", outer="reliable")

    ms, (st, r) = _time_solves(torch, reliable64, reps)
    record("fp64_reliable", ms, r.inner_iterations, r.fp64_applies,
           (8 + r.inner_iterations * CG64_BYTES_PER_IT + r.outer_iterations * RELIABLE_UPDATE_BYTES + RESID_BYTES) * n,
           {"status": st, "corrections": r.outer_iterations,
            "solver": "FP64 CG with reliable updates (true residual recomputed in FP64), true 1e-10"})
    x_rel = x.clone()

    def flexible(tol=inner_tol):
        x.zero_()
        return op.solve_mixed(x, b, inner_tol=tol, outer_tol=1e-10, outer="flexible")

    for name, tol in (("mixed", inner_tol), ("mixed_inner_1e-5", 1e-5)):
        ms, (st, r) = _time_solves(torch, lambda: flexible(tol), reps)
        record(name, ms, None, r.fp64_applies,
               (8 + RESID_BYTES * (r.fp64_applies - r.outer_iterations) + r.inner_iterations * FP32_INNER_BYTES_PER_IT
                + r.outer_iterations * FLEX_OUTER_BYTES) * n,
               {"status": st, "inner_tol": tol, "outer_steps": r.outer_iterations,
                "inner_iterations": r.inner_iterations, "fp64_applies": r.fp64_applies,
                "rel_residual_reported": r.rel_residual,
                "rel_diff_vs_fp64_reliable": float(((x - x_rel).norm() / x_rel.norm()).item()),
                "rel_diff_vs_fp64_cg": float(((x - x_ref).norm() / x_ref.norm()).item()),
                "solver": "flexible CG in FP64, inner CG in FP32 (values and accumulation) to relative %g" % tol})
    m = arms["mixed"]
    out = {"workload": "%dx%d quads, p=%d (%d DoF), pen %g, f = 8 pi^2 sin(2 pi x) sin(2 pi y), x0 = 0, "
                       "true relative residual 1e-10" % (dim, dim, p, n, pen),
           "solves_per_s": m["solves_per_s"], "ms": m["ms"], "true_rel_residual": m["true_rel_residual"],
           "L2_over_fp64_L2": m["L2"] / arms["fp64_reliable"]["L2"],
           "speedup_vs_fp64_reliable": arms["fp64_reliable"]["ms"] / m["ms"],
           "speedup_vs_fp64_cg": arms["fp64_cg"]["ms"] / m["ms"], "arms": arms,
           "timing": "CUDA events around each solve call, median of %d after one untimed solve" % reps}
    if cpu:
        import oracle_lib

        orc = oracle_lib.load()
        nthreads = os.cpu_count() or 1
        bn = b.cpu().numpy()
        k = 4
        orc.cg(p, dim, pen, bn, 0.0, max_it=1, nthreads=nthreads)  # warm-up
        t0 = time.perf_counter()
        orc.cg(p, dim, pen, bn, 0.0, max_it=k, nthreads=nthreads)
        per_it = (time.perf_counter() - t0) / k
        its = arms["fp64_cg"]["iterations"]
        out["cpu_baseline"] = {"value": 1.0 / (per_it * its), "unit": "solves/s", "cores": nthreads, "kind": "port",
                               "sample": "%d CG iterations of the oracle (the reference's CG and matvec restated in "
                                         "C) on the same problem, %.2f s per iteration, scaled to the %d iterations "
                                         "of the FP64 solve" % (k, per_it, its)}
    op.close()
    return out


def solve16_metrics(torch, sipg, steps=20, warmup=3, cpu=True, hsweep=False):
    """The 16 x 16, p = 4 solve to relative residual 1e-12 (one solve per step),
    end to end from a host right-hand side to a host solution."""
    import numpy as np

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

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    wall = (time.perf_counter() - t0) / steps
    dev_ms = []
    for _ in range(5):
        x.zero_()
        dev_ms.append(op.cg(x, b_dev, 1e-12, relative=True)[1].time_ms)
    dev_ms.sort()
    r = res["r"]
    l2, h1, mx = op.err_norms("sinsin", x)
    out = {"workload": "16x16 quads, p=4 (6400 DoF), pen 16, f = 8 pi^2 sin(2 pi x) sin(2 pi y), x0 = 0, CG to "
                       "relative residual 1e-12",
           "solves_per_s": 1e3 / dev_ms[2], "device_ms_per_solve": dev_ms[2], "iterations": r.iterations,
           "true_rel_residual": _true_rel(op, x, b_dev), "L2": l2, "H1": h1, "max_err": mx,
           "e2e": {"value": 1.0 / wall, "unit": "solves/s", "h2d_bytes_per_step": op.ndof * 8,
                   "d2h_bytes_per_step": op.ndof * 8, "api": "sipg_cg_f64 with host b in, host x out"},
           "roofline": _roofline_solve((8 + RESID_BYTES + r.iterations * CG64_BYTES_PER_IT) * op.ndof, dev_ms[2],
                                       r.iterations, op.ndof, p, None)}
    out["roofline"]["note"] = "6400 DoF (51 KB per vector) stay in L2: latency-bound, not HBM-bound"
    try:
        import oracle_lib

        if oracle_lib.ref_gpu_available():
            xr = torch.zeros_like(b_dev)
            it, ms = oracle_lib.ref_gpu().cg(p, dim, pen, xr.data_ptr(), b_dev.data_ptr(),
                                             1e-12 * float(b_dev.norm().item()))
            out["reference_kernels_same_gpu"] = {"iterations": it, "ms_per_solve": ms, "solves_per_s": 1e3 / ms,
                                                 "source": "reference kernels + its CG loop (cuBLAS dots)"}
    except Exception as exc:
        out["reference_kernels_same_gpu"] = {"unavailable": str(exc)}
    if cpu:
        import oracle_lib

        orc = oracle_lib.load()
        bn = b_dev.cpu().numpy()
        best = None
        for nthreads in sorted({1, os.cpu_count() or 1}):
            t0 = time.perf_counter()
            reps = 0
            while reps < 3 or time.perf_counter() - t0 < 1.0:
                it, _, _ = orc.cg(p, dim, pen, bn, 1e-12, rel=True, nthreads=nthreads)
                reps += 1
            v = reps / (time.perf_counter() - t0)
            row = {"value": v, "unit": "solves/s", "cores": nthreads, "kind": "port",
                   "sample": "%d solves of %d iterations each" % (reps, it)}
            out.setdefault("cpu_by_threads", []).append(row)
            if best is None or v > best["value"]:
                best = row
        out["cpu_baseline"] = dict(best, note="the fastest thread count of 1 and all %d host threads (6400 DoF: "
                                              "threading overhead can exceed the work)" % (os.cpu_count() or 1))
    if hsweep:
        # h-convergence over dim = 4..512 (p = 4, same problem, pen p^2, CG to
        # 1e-12 relative): error norms and their rates log2(e(h) / e(h/2))
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
        out["h_convergence_p4"] = hs
    op.close()
    return out


def run_solve16(args):
    import torch

    import sipg_gb300 as sipg

    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    m = solve16_metrics(torch, sipg, args.steps, args.warmup, cpu=not args.no_cpu_baseline, hsweep=True)
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    extra = {k: v for k, v in m.items() if k not in ("workload", "solves_per_s")}
    line = _base_line(args, "solves/s, 16x16 quads p=4 SIPG-SEM Poisson CG to relative residual 1e-12",
                      m["solves_per_s"], "solves/s", True, "f64", {"workload": m["workload"]},
                      clocks=clocks, gpu_launches=launches, **extra)
    print(json.dumps(line), flush=True)
    return 0


def run_mixed(args):
    """512 x 512, p = 6: the mixed-precision solve vs the FP64 solvers, all to a
    true relative residual of 1e-10 (the reference's CG reports its own)."""
    import torch

    import sipg_gb300 as sipg

    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    fp64_peak, _ = sipg.probe_fma_peak()
    m = mixed_metrics(torch, sipg, reps=max(3, min(args.steps, 5)), cpu=not args.no_cpu_baseline,
                      fp64_peak=fp64_peak)
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    extra = {k: v for k, v in m.items() if k not in ("workload", "solves_per_s")}
    line = _base_line(args, "solves/s to true relative residual 1e-10, 512x512 quads p=6, mixed precision "
                            "(FP32 inner CG, FP64 flexible CG)", m["solves_per_s"], "solves/s", True,
                      "f32 (inner) + f64 (outer)", {"workload": m["workload"]}, clocks=clocks,
                      gpu_launches=launches, **extra)
    print(json.dumps(line), flush=True)
    return 0


def _batch_case(torch, sipg, workloads, probs, cpu=True):
    """Batched mixed solve of `probs` [(dim, p, pen, modes)] (flexible CG in
    FP64 around an FP32 inner CG, every problem to a true relative residual of
    1e-10) vs the same solves one at a time with the plain FP64 CG (relative
    1e-10 on its recursive residual; its true residuals are reported)."""
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
    true_b = max(_true_rel(batch.op(k), xs[k], bs[k]) for k in range(len(probs)))
    # one at a time, plain FP64 CG (operators reused across equal problems)
    ops = {}
    t_seq = 0.0
    worst = 0.0
    true_64 = 0.0
    its64 = []
    for k, (d, p, pen, _) in enumerate(probs):
        key = (d, p, pen)
        if key not in ops:
            ops[key] = sipg.Operator(d, p, pen)
        x = torch.zeros_like(bs[k])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, r64 = ops[key].cg(x, bs[k], 1e-10, relative=True)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t0
        its64.append(r64.iterations)
        true_64 = max(true_64, _true_rel(ops[key], x, bs[k]))
        worst = max(worst, float(((xs[k] - x).norm() / max(x.norm().item(), 1e-300)).item()))
    for op in ops.values():
        op.close()
    n = len(probs)
    dofs = [workloads.ndof(d, p) for d, p, _, _ in probs]
    bytes_b = sum(nk * (8 + FP32_INNER_BYTES_PER_IT * r.inner_iterations + FLEX_OUTER_BYTES * r.outer_iterations +
                        RESID_BYTES * (r.fp64_applies - r.outer_iterations)) for nk, r in zip(dofs, res))
    bytes_64 = sum(nk * (8 + RESID_BYTES + CG64_BYTES_PER_IT * it) for nk, it in zip(dofs, its64))
    peak, src = measured_peaks()
    out = {"problems": n, "status": st, "converged": ok, "batch_solves_per_s": n / t_batch,
           "fp64_one_at_a_time_solves_per_s": n / t_seq, "speedup": t_seq / t_batch,
           "max_true_rel_residual_batch": true_b, "max_true_rel_residual_fp64_cg": true_64,
           "max_rel_diff_vs_fp64": worst, "total_dof": sum(dofs),
           "inner_iterations_max": max(r.inner_iterations for r in res),
           "outer_steps_max": max(r.outer_iterations for r in res),
           "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak,
                        "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % src,
                        "batch_achieved": bytes_b / t_batch / 1e9, "batch_frac": bytes_b / t_batch / 1e9 / peak,
                        "fp64_achieved": bytes_64 / t_seq / 1e9, "fp64_frac": bytes_64 / t_seq / 1e9 / peak},
           "timing": "wall clock around each whole batch / solve, synchronised"}
    if cpu:
        import oracle_lib

        orc = oracle_lib.load()
        nthreads = os.cpu_count() or 1
        kbig = max(range(n), key=lambda k: dofs[k])
        d, p, pen, _ = probs[kbig]
        bn = bs[kbig].cpu().numpy()
        t0 = time.perf_counter()
        orc.cg(p, d, pen, bn, 0.0, max_it=4, nthreads=nthreads)
        per_dof_it = (time.perf_counter() - t0) / 4 / dofs[kbig]
        est = sum(nk * it for nk, it in zip(dofs, its64)) * per_dof_it
        out["cpu_baseline"] = {"value": n / est, "unit": "solves/s", "cores": nthreads, "kind": "port",
                               "sample": "4 oracle CG iterations on the largest problem (%dx%d, p=%d), %.3g s per "
                                         "DoF-iteration, scaled to every problem's FP64 iteration count" %
                                         (d, d, p, per_dof_it)}
    batch.close()
    return out


def run_batch(args):
    import torch

    import sipg_gb300 as sipg
    import workloads

    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    cpu = not args.no_cpu_baseline
    a = _batch_case(torch, sipg, workloads, workloads.shared_mesh_rhs(64, 256, 4, seed=1), cpu)
    b = _batch_case(torch, sipg, workloads, workloads.uneven_problems(args.uneven, seed=2), cpu)
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    line = _base_line(args, "solves/s, batched mixed-precision solves to 1e-10 (64 RHS on 256x256 p=4)",
                      a["batch_solves_per_s"], "solves/s", True, "f32 (inner) + f64 (outer)",
                      {"workload": "(a) 64 RHS, 256x256 quads p=4, 4 sine modes each (seed 1); "
                                   "(b) %d problems, N log-uniform [16,256], p in 2..8 (seed 2)" % args.uneven},
                      shared_mesh=a, uneven=b, clocks=clocks, gpu_launches=launches)
    print(json.dumps(line), flush=True)
    return 0


def _serve_stream(sipg, reqs, precision, max_active=256, budget=150 << 30):
    """Replays `reqs` [(t_arrival_s, dim, p, pen, modes, tol)] against one
    server in real time: each request is submitted once the wall clock passes
    its arrival time, the host steps the server and polls results between
    arrivals.  Latency = submit -> retirement (the server's own clock)."""
    srv = sipg.Server(budget_bytes=budget, max_active=max_active, iters_per_step=8)
    pending = list(reqs)
    inflight = {}
    lat, failed = [], 0
    algo_bytes = 0.0  # algorithmic HBM bytes of the completed solves
    dof_its = 0.0     # sum of DoF x iterations (FP64: CG iterations)
    peak_bytes = 0
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
        peak_bytes = max(peak_bytes, srv.stats().bytes_in_use)
        for rid in list(inflight):
            r = srv.poll(rid)
            if r.done:
                if r.status == 0:
                    lat.append(r.latency_ms)
                    _, d, p, _, _, _ = pending[inflight[rid]]
                    nk = d * d * (p + 1) * (p + 1)
                    if precision == sipg.F64:
                        algo_bytes += nk * (8 + RESID_BYTES + CG64_BYTES_PER_IT * r.iterations)
                    else:
                        algo_bytes += nk * (8 + RESID_BYTES + FP32_INNER_BYTES_PER_IT * r.iterations +
                                            FLEX_OUTER_BYTES * r.corrections)
                    dof_its += nk * r.iterations
                else:
                    failed += 1
                srv.release(rid)
                del inflight[rid]
    wall = time.perf_counter() - t0
    setup_ms, prep_ms = srv.stats().setup_ms, srv.stats().prep_ms
    srv.close()
    lat.sort()
    q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))] if lat else None
    peak, src = measured_peaks()
    return {"requests": len(reqs), "completed": len(lat), "failed": failed, "wall_s": wall,
            "solves_per_s": len(lat) / wall, "p50_ms": q(0.5), "p99_ms": q(0.99), "max_ms": lat[-1] if lat else None,
            "peak_bytes_in_use": peak_bytes, "budget_bytes": budget,
            "arrival_span_s": reqs[-1][0] if reqs else 0.0,
            "admission_setup_s": setup_ms / 1e3,
            "background_prep_s": prep_ms / 1e3,
            "dof_iterations": dof_its,
            "roofline": {"bound": "hbm", "achieved": algo_bytes / wall / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo_bytes / wall / 1e9 / peak, "algorithmic_bytes": algo_bytes,
                         "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % src,
                         "note": "over the stream's wall time, arrival gaps included: the server's use of HBM, "
                                 "not one kernel's efficiency"}}


def serve_metrics(sipg, workloads, rate, count, cpu=True):
    """The first `count` requests of the seed-3 stream at `rate` requests/s,
    served once with every request mixed precision and once plain FP64; the
    CPU baseline is the oracle's CG on all host cores, its cost per DoF and
    iteration measured on one 256 x 256, p = 4 problem and scaled to the
    FP64 arm's iteration counts."""
    reqs = workloads.request_stream(count=count, rate=rate, seed=3)
    out = {"rate_per_s": rate, "requests": count,
           "stream": "the first %d of the 10,000-request stream (seed 3): Poisson arrivals at %g/s, N log-uniform "
                     "[8,512], p in 2..8, tol in {1e-8, 1e-10}, 150 GB budget" % (count, rate),
           "mixed": _serve_stream(sipg, reqs, sipg.F32), "fp64": _serve_stream(sipg, reqs, sipg.F64)}
    if cpu and out["fp64"]["completed"]:
        import numpy as np

        import oracle_lib

        orc = oracle_lib.load()
        nthreads = os.cpu_count() or 1
        d, p = 256, 4
        b = np.random.default_rng(0).uniform(-1.0, 1.0, d * d * (p + 1) ** 2)
        t0 = time.perf_counter()
        orc.cg(p, d, float(p * p), b, 0.0, max_it=4, nthreads=nthreads)
        per_dof_it = (time.perf_counter() - t0) / 4 / b.size
        est = out["fp64"]["dof_iterations"] * per_dof_it
        out["cpu_baseline"] = {"value": out["fp64"]["completed"] / est, "unit": "solves/s", "cores": nthreads,
                               "kind": "port",
                               "sample": "4 oracle CG iterations on 256x256, p=4 (%.3g s per DoF-iteration), "
                                         "scaled to the FP64 arm's iterations of every request" % per_dof_it}
    return out


def run_serve(args):
    """The request stream at the given arrival rates, mixed-precision requests
    and plain FP64 requests through the same server."""
    import sipg_gb300 as sipg
    import workloads

    rates = [float(r) for r in str(args.rate).split(",")]
    sampler = ClockSampler(0)
    sampler.start()
    n0 = sipg.launch_count()
    sweep = [serve_metrics(sipg, workloads, rate, args.requests, cpu=(k == 0 and not args.no_cpu_baseline))
             for k, rate in enumerate(rates)]
    launches = sipg.launch_count() - n0
    clocks = sampler.stop()
    head = sweep[0]
    line = _base_line(args, "p99 latency (ms), solve server, mixed precision, at %g requests/s" % head["rate_per_s"],
                      head["mixed"]["p99_ms"], "ms", False, "f32 (inner) + f64 (outer)",
                      {"workload": "%d requests per rate, Poisson arrivals, N log-uniform [8,512], p in 2..8, "
                                   "tol in {1e-8, 1e-10} (seed 3); 150 GB budget" % args.requests},
                      sweep=sweep, clocks=clocks, gpu_launches=launches)
    print(json.dumps(line), flush=True)
    return 0


PROFILE_CASES = ("apply_f64_1024_p4", "apply_f32_1024_p4", "apply_f32_571_p6", "apply_pairs_512_p6",
                 "mixed_512_p6", "cg_512_p6", "pcg_512_p6", "cg_16_p4")


def run_profile_case(name, reps=4):
    """A small, bounded run of one kernel path for an ncu capture (one GPU, a
    few launches of each kernel, at most a few GB on the device).  Prints one
    line; the numbers it prints are not bench values."""
    import numpy as np
    import torch

    import sipg_gb300 as sipg

    torch.cuda.set_device(0)
    kind, dim, p = name.split("_")[0], int(name.split("_")[-2]), int(name.split("_")[-1][1:])
    if name.startswith("apply_pairs"):
        kind = "pairs"
    elif name.startswith("apply_f32"):
        kind = "f32"
    elif name.startswith("apply_f64"):
        kind = "f64"
    op = sipg.Operator(dim, p, float(p * p))
    info = {"case": name, "ndof": op.ndof}
    if kind in ("f64", "f32", "pairs"):
        x = torch.from_numpy(np.random.default_rng(0).uniform(-1.0, 1.0, op.ndof)).cuda()
        if kind == "f32":
            x = x.float()
        if kind == "pairs":
            x = sipg.to_pairs(x)
        y = torch.empty_like(x)
        f = op.apply_pairs if kind == "pairs" else op.apply
        for _ in range(reps):
            f(x, y)
    else:
        b = op.rhs("sinsin")
        x = torch.zeros_like(b)
        if kind == "mixed":
            st, r = op.solve_mixed(x, b, inner_tol=MIXED_INNER_TOL, outer_tol=1e-10, outer="flexible")
            info.update(status=st, outer=r.outer_iterations, inner=r.inner_iterations)
        elif kind == "cg":
            st, r = op.cg(x, b, 1e-10, relative=True, max_it=0 if dim <= 64 else 40)
            info.update(status=st, iterations=r.iterations)
        elif kind == "pcg":
            st, r = op.pcg(x, b, 1e-10, relative=True, max_it=40)
            info.update(status=st, iterations=r.iterations)
    torch.cuda.synchronize()
    op.close()
    print(json.dumps(info), flush=True)
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
    ap.add_argument("--requests", type=int, default=1000, help="serve: requests per arrival rate")
    ap.add_argument("--rate", default="50,200,2000", help="serve: arrival rates per second, comma-separated")
    ap.add_argument("--serve-requests", type=int, default=300,
                    help="default line: requests of the serving stream at 50/s (a prefix of the 10,000)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="default line: skip the mixed, serve and solve16 keys")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", choices=PROFILE_CASES, default=None,
                    help="run one small kernel case for an ncu capture (no JSON bench line)")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args.profile_case)
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
