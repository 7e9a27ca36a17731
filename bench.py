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
# DFMA-pipe instructions per DoF issued by the fused FP64 kernel (column form):
# volume + lifting 2n + 6, face derivatives 4, face combine and corrections ~ 16/n
FP64_FLOPS_PER_DOF = 2.0 * (2 * (DEGREE + 1) + 10 + 16.0 / (DEGREE + 1))
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
    ms = e0.elapsed_time(e1)
    if pg:
        t = torch.tensor([ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
        pg.barrier()
    ms_per_step = ms / args.steps
    value = world * args.steps * APPLIES_PER_STEP * NDOF / (ms * 1e-3) / 1e9

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
    e2e_s = time.perf_counter() - t0
    if pg:
        t = torch.tensor([e2e_s], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * e2e_steps * NDOF / e2e_s / 1e9
    ok = bool(np.array_equal(h_out.numpy(), y.cpu().numpy()))

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
                "matches_device_result": ok},
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
