"""Benchmark of the GB300 annealing backend on the 100k-qubit FP32 configuration.

Workload: random 3-regular graph, n = 100,000 (seeded), J in {-1,+1}, h ~ U(-0.5, 0.5),
200 Trotter steps over T = 20, bond dim 16, BP tolerance 1e-5 with at most 50 sweeps,
complex64 arithmetic.  A "step" is one annealing step (simple update + Rz/Rx layers +
symmetric gauge + BP to tolerance), taken in the saturated regime: the anneal is first run
(untimed) until the bond dimension reaches 16, then W warm-up steps and K timed steps
continue the schedule.  Inputs (6.6 GB of node tensors, 0.6 GB of messages) are resident
in HBM and far larger than L2, so no L2 flush is needed between steps.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference] [--n N]

--impl reference times the reference algorithm's CPU implementation (the numpy oracle
port, FP64 like the reference's default) on a bounded sample: a 200-node instance of the
same generator, annealed to the same saturated regime (bond dim 16, reached at the same
step as the 100k-node job), then W warm-up and K timed steps of the same schedule window,
scaled to 100k nodes by the node count (all per-step work is per node).  The GPU arm's
cpu_baseline runs the same function with the same K and W.
Under torchrun (N > 1) every rank runs an independent replica job on its own GPU
(the step is not sharded across GPUs here: replicas only); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import logging
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "anneal steps/s & BP msg-updates/s at stated <Z> err vs FP64; p50/p99 job latency"
WORKLOAD = "random 3-regular n={n} (seed 0), J=+-1, h~U(-0.5,0.5), chi={chi}, T=20, 200 steps, bp_eps 1e-5, <=50 sweeps"
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
SAMPLE_N = 200


# executed / algorithmic FLOPs of the degree-3 message kernels: the shape-specialised schedule
# (3 products + 3 closing contractions) against the reference order (6 + 3)
# Executed share of the reference order's FLOPs in the degree-3 half-node sweep: 3 bond products
# and 3 closing contractions (Hermitian split) instead of 6 + 3, each closing contraction forming
# only the NG (NG + 1) / 2 upper 4x4 tiles of its NG x NG tile grid (NG = chi / 4).
EXECUTED_FRACTION = {c: (3 + 3 * ((c // 4) * (c // 4 + 1) / 2) / (c // 4) ** 2) / 9 for c in (4, 8, 12, 16)}

# DRAM bytes one chi-16 degree-3 BP sweep moves per node: ncu captures of a 10k-node sweep,
# half-node kernel + bp_combine_kernel 224.9 MB (the work is per node): the tensor-core kernel
# tcx_half_kernel_d3c16 830.1 MB, the CUDA-core kernel tiled_half_kernel<3,16> 829.2 MB.
SWEEP_DRAM_BYTES_PER_NODE = {"tensor": (830.11e6 + 224.94e6) / 10000, "cuda-core": (829.23e6 + 224.94e6) / 10000}
# FLOPs the tensor cores execute per degree-3 bond-dim-16 node in the 2xFP16 kernel: per half-node
# 36 product MMAs of 128 x 32 x 16 and 96 closing MMAs of 64 x 32 x 16 (2 FLOP per MAC)
TC_EXECUTED_FLOPS_PER_NODE = 2 * (36 * 128 * 32 * 16 + 96 * 64 * 32 * 16) * 2


def peaks() -> tuple[dict, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        with open(p) as f:
            return json.load(f), "measured"
    return FALLBACK_PEAKS, "fallback"


def fp32_peak_tflops(dev) -> float:
    """FP32 FMA throughput of this GPU (bqa_fp32_fma_probe: 16 independent FMA chains per
    thread, 8 CTAs of 256 per SM), median of 5 timed launches after 2 untimed."""
    import torch
    from bqa_gb300 import _lib
    probes = _lib.load_probes()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = 8 * sms, 4000
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    ts = []
    for i in range(7):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        if probes.bqa_fp32_fma_probe(blocks, iters, out.data_ptr(), st.cuda_stream) != 0:
            raise RuntimeError("bqa_fp32_fma_probe failed")
        b.record(st)
        torch.cuda.synchronize(dev)
        if i >= 2:
            ts.append(a.elapsed_time(b))
    flops = 2.0 * 16 * iters * blocks * 256
    return flops / (float(np.median(ts)) / 1e3) / 1e12


def mma_peak_tflops(dev, kind: int) -> float:
    """Warp-level mma.sync throughput (bqa_mma_probe; kind 0 bf16 m16n8k16, 1 tf32 m16n8k8), 8
    CTAs of 256 per SM, best of 5 timed launches after 1 untimed."""
    import torch
    from bqa_gb300 import _lib
    probes = _lib.load_probes()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = 8 * sms, 2000
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    ts = []
    for i in range(6):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        if probes.bqa_mma_probe(kind, blocks, iters, out.data_ptr(), st.cuda_stream) != 0:
            raise RuntimeError("bqa_mma_probe failed")
        b.record(st)
        torch.cuda.synchronize(dev)
        if i >= 1:
            ts.append(a.elapsed_time(b))
    flops = 2.0 * 16 * 8 * (16 if kind == 0 else 8) * 8 * iters * blocks * 8
    return flops / (min(ts) / 1e3) / 1e12


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(steps: int, warmup: int, n_full: int, chi: int, dtype=None) -> dict:
    """Time the oracle port of the reference algorithm on the bounded sample, in the same regime
    as the GPU arm: a SAMPLE_N-node instance of the benchmark generator is annealed from the
    start of the schedule until its bond dim reaches ``chi`` (untimed; it saturates at the same
    step as the 100k-node job), then ``warmup`` untimed and ``steps`` timed steps continue the
    schedule.  The gate layer (simple update, Rz, Rx, symmetric gauge) and the BP run are timed
    apart, so the line also gives the time per BP sweep and the step rate at any sweep count."""
    import logging as _logging
    from bqa_gb300 import instances
    from oracle import bqa_oracle as orc
    _logging.getLogger("oracle.bqa_oracle").setLevel(_logging.ERROR)
    dtype = np.complex128 if dtype is None else dtype
    octx = orc.make_context(instances.headline_gpu_job(n=SAMPLE_N, seed=0, chi=chi), dtype=dtype)
    st = orc.initialize_state(octx)
    sched = [i for i in octx.instructions if isinstance(i, dict)]
    t_prep = time.perf_counter()
    s = 0
    while s < len(sched) - 1 and (st.bond_dim < chi or s == 0):
        orc.run_layer(octx, sched[s]["xtime"], sched[s]["ztime"], st)
        s += 1
    prep_steps, prep_s = s, time.perf_counter() - t_prep

    def step(i, timed):
        ins = sched[min(i, len(sched) - 1)]
        t0 = time.perf_counter()
        orc.simple_update(octx, ins["ztime"], st)
        orc.apply_z_layer(octx, ins["ztime"], st)
        orc.apply_x_layer(ins["xtime"], st)
        orc.set_to_symmetric_gauge(octx, st)
        t1 = time.perf_counter()
        sw = orc.run_bp(octx, st)
        t2 = time.perf_counter()
        return (t1 - t0, t2 - t1, sw) if timed else None

    for i in range(warmup):
        step(s + i, False)
    s += warmup
    rec = [step(s + i, True) for i in range(steps)]
    gate = sum(r[0] for r in rec)
    bp = sum(r[1] for r in rec)
    sweeps = sum(r[2] for r in rec)
    scale = SAMPLE_N / n_full
    sample_rate = steps / (gate + bp)
    per_sweep = bp / max(sweeps, 1)
    return {
        "value": sample_rate * scale,
        "unit": "steps/s",
        "cores": len(os.sched_getaffinity(0)),
        "blas_threads": os.environ.get("OPENBLAS_NUM_THREADS", "library default"),
        "kind": "port",
        "scale": scale,
        "sweeps_per_step": sweeps / steps,
        "gate_layer_s_per_step": gate / steps,
        "bp_sweep_s": per_sweep,
        "bp_msg_updates_per_s": octx.edges_number / per_sweep,
        "sample": (f"reference algorithm (numpy oracle port, {np.dtype(dtype).name}) on a {SAMPLE_N}-node instance of the "
                   f"same generator, annealed from step 0 until its bond dim reached {chi} (step {prep_steps}, "
                   f"{prep_s:.1f} s untimed), then {warmup} untimed and {steps} timed steps of the schedule: "
                   f"{gate + bp:.1f} s ({sample_rate:.3f} steps/s; gate layer {gate / steps:.3f} s/step, "
                   f"{sweeps / steps:.1f} BP sweeps/step at {per_sweep:.3f} s/sweep), scaled by {SAMPLE_N}/{n_full} "
                   f"nodes (all per-step work is per node); batched small matmuls run effectively on one core"),
    }


def cpu_rate_at(cpu: dict, sweeps_per_step: float) -> float:
    """Steps/s of the CPU baseline at another BP sweep count per step (full-size, scaled)."""
    return cpu["scale"] / (cpu["gate_layer_s_per_step"] + sweeps_per_step * cpu["bp_sweep_s"])


ACCURACY_FIXTURE = ROOT / "tests" / "golden" / "c2_rr3_n10k_chi16.npz"


def measured_accuracy(mixed: bool = False) -> dict | None:
    """<Z> / Bloch-vector error of the complex64 path against the reference at FP64, measured in
    this run: the 10,000-node instance of this workload's generator (chi 16, the first 66 steps
    of the 200-step schedule, past saturation) through bqa_gb300.run_qa, compared with the
    reference's Bloch vectors recorded in the fixture."""
    if not ACCURACY_FIXTURE.exists():
        return None
    import bqa_gb300
    from tests.golden.make_golden_c2 import config_from_fixture
    conf = config_from_fixture(ACCURACY_FIXTURE)
    want = np.load(ACCURACY_FIXTURE)["bloch"]
    saved = {k: os.environ.get(k) for k in ("BQA_PRECISION", "BQA_GB300_MIXED")}
    os.environ["BQA_PRECISION"] = "single"
    os.environ["BQA_GB300_MIXED"] = "1" if mixed else "0"
    try:
        t0 = time.perf_counter()
        got = bqa_gb300.run_qa(dict(conf), as_arrays=True)[0][1]
        secs = time.perf_counter() - t0
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    err = np.abs(got - want)
    return {"bloch_err_max": float(err.max()), "z_err_max": float(err[:, 2].max()),
            "z_err_mean": float(err[:, 2].mean()), "seconds": round(secs, 1),
            "where": ("mixed-precision " if mixed else "") +
                     "complex64 path vs the reference at FP64 (fixture tests/golden/c2_rr3_n10k_chi16.npz: "
                     "10,000-node instance of this generator, chi 16, first 66 steps, past saturation), "
                     "measured in this run through bqa_gb300.run_qa"}


def run_reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    base = cpu_reference(args.steps, args.warmup, args.n, args.chi)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 / base["value"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD.format(n=args.n, chi=args.chi)},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def max_over_ranks(values: list, device=None) -> list:
    """Element-wise maximum of ``values`` over the ranks of the default process group (the
    slowest replica's times define the job's time); the values themselves without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def replica_value(world: int, steps: int, t_max_ms: float) -> float:
    """Whole-job steps/s of ``world`` independent replicas that each ran ``steps`` steps, the
    slowest in ``t_max_ms``."""
    return world * steps / (t_max_ms / 1000.0)


def launch_count() -> int:
    """Kernel launches the backend library has issued so far (bqa_launch_count; the timed steps
    run Python-driven, without graphs, so every launch counts)."""
    from bqa_gb300 import _lib
    return int(_lib.load().dll.bqa_launch_count())


def run_gpu_arm(args) -> None:
    import torch
    import torch.distributed as dist
    from bqa_gb300 import instances
    from bqa_gb300.engine import Annealer
    from bqa_gb300.layout import build_context

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    def barrier():
        if world > 1:
            dist.barrier()

    conf = instances.headline_gpu_job(n=args.n, seed=0, chi=args.chi)
    ctx = build_context(conf)
    steps_all = [i for i in ctx.instructions if isinstance(i, dict)]
    job = Annealer(ctx, device=dev, precision="single")

    # untimed: anneal until the bond dimension saturates
    t_prep = time.perf_counter()
    s = 0
    while s < len(steps_all) - 1 and (job.bond_dim < args.chi or s == 0):
        job.run_layer(steps_all[s]["xtime"], steps_all[s]["ztime"])
        s += 1
    prep_steps, prep_s = s, time.perf_counter() - t_prep

    def step_at(i):
        ins = steps_all[min(i, len(steps_all) - 1)]
        return ins["xtime"], ins["ztime"]

    for i in range(args.warmup):
        job.run_layer(*step_at(s + i))
    s += args.warmup

    # the end-to-end pass below replays the timed steps from this state
    snap = job.snapshot()
    s_timed = s

    # timed region: K steps, device-timed with CUDA events on the launch stream
    job.enable_kernel_timing(True)
    job.stats.clear()
    barrier()
    torch.cuda.synchronize(dev)
    launches0 = launch_count()
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clocks:
        # profilers select the timed steps by this range (ncu --nvtx --nvtx-include "timed_steps/")
        torch.cuda.nvtx.range_push("timed_steps")
        ev0.record(stream)
        for i in range(args.steps):
            job.run_layer(*step_at(s + i))
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        torch.cuda.nvtx.range_pop()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = launch_count() - launches0
    s += args.steps
    kt = job.kernel_times()
    job.enable_kernel_timing(False)
    window = list(job.stats)

    # end to end through the step API with host results, over the same K steps from the same
    # state: per step the instruction goes in by value, the new marginals of every qubit come
    # back to host memory
    job.restore(snap)
    del snap
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for i in range(args.steps):
        job.run_layer(*step_at(s_timed + i))
        bloch = job.bloch_vectors()
    e2e_s = time.perf_counter() - t0

    # the mixed-precision form (BF16 tensor-core sweeps while the BP distance is above the
    # switch, FP32 sweeps to the tolerance) over the same schedule window, from its own anneal
    mixed = None
    if args.mixed:
        mjob = Annealer(ctx, device=dev, precision="single", mixed=True)
        sm = 0
        while sm < len(steps_all) - 1 and (mjob.bond_dim < args.chi or sm == 0):
            mjob.run_layer(steps_all[sm]["xtime"], steps_all[sm]["ztime"])
            sm += 1
        for i in range(args.warmup):
            mjob.run_layer(*step_at(sm + i))
        sm += args.warmup
        mjob.enable_kernel_timing(True)
        mjob.stats.clear()
        barrier()
        torch.cuda.synchronize(dev)
        mlaunches0 = launch_count()
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0.record(stream)
        for i in range(args.steps):
            mjob.run_layer(*step_at(sm + i))
        m1.record(stream)
        torch.cuda.synchronize(dev)
        mlaunches = launch_count() - mlaunches0
        barrier()
        mms = m0.elapsed_time(m1)
        mkt = mjob.kernel_times()
        mjob.enable_kernel_timing(False)
        msplit: dict = {}
        for name, t, _, _ in mkt:
            msplit[name] = msplit.get(name, 0.0) + t
        mixed = {"ms_raw": mms, "sweeps_per_step": float(np.mean([w["sweeps"] for w in mjob.stats])),
                 "time_split_ms": {k: round(v, 2) for k, v in sorted(msplit.items(), key=lambda kv: -kv[1])},
                 "gpu_launches": mlaunches}
        del mjob
        torch.cuda.empty_cache()

    t_max, e2e_s = max_over_ranks([ms, e2e_s], device=dev)
    if mixed is not None:
        mixed["ms_raw"] = max_over_ranks([mixed["ms_raw"]], device=dev)[0]
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    value = replica_value(world, args.steps, t_max)
    sweep_ev = [k for k in kt if k[0] == "bp_sweep"]
    bp_ms = sum(k[1] for k in sweep_ev)
    bp_flops = sum(k[2] for k in sweep_ev)
    bp_bytes = sum(k[3] for k in sweep_ev)
    sweeps = [w["sweeps"] for w in window]
    by_name: dict = {}
    for name, t, _, _ in kt:
        by_name[name] = by_name.get(name, 0.0) + t
    pk, pk_kind = peaks()
    fp32_peak = fp32_peak_tflops(dev)
    achieved = bp_flops / (bp_ms / 1000.0) / 1e12 if bp_ms > 0 else 0.0
    cpu = cpu_reference(args.steps, args.warmup, args.n, args.chi) if not args.no_cpu_baseline else None
    if cpu is not None:
        cpu["at_gpu_sweeps_per_step"] = {"sweeps_per_step": float(np.mean(sweeps)),
                                         "value": cpu_rate_at(cpu, float(np.mean(sweeps))), "unit": "steps/s"}
        # the reference's BQA_PRECISION=single arithmetic, a shorter window (the FP32 ratio)
        single = cpu_reference(min(args.steps, 5), 1, args.n, args.chi, dtype=np.complex64)
        cpu["single"] = {k: single[k] for k in ("value", "unit", "sweeps_per_step", "gate_layer_s_per_step",
                                                "bp_sweep_s", "sample")}
    n_el = ctx.nodes_number
    accuracy = measured_accuracy()
    # serving: a bounded Poisson stream of small jobs through the continuous-batching server
    serving = None
    if args.serve_jobs > 0:
        wide = args.serve_stream == "wide"
        serving = {"stream": SERVING_STREAM_WIDE if wide else SERVING_STREAM,
                   **serving_measurement(args.serve_jobs, args.rate, wide=wide)}
    # the other configurations' shapes, short: the mixed-degree job at bond dim 4 (every node in
    # shared memory) and the degree-4 bond-dim-32 sweep (global-memory kernels)
    tuned = [job.plans[c].describe() for c in sorted(job.plans)] if job.autotune else "off"
    # the (3, 16) message kernel the timed sweeps ran: the tuner's choice, else the library default
    if job.autotune and 16 in job.plans:
        tensor_sweep = "tensor" in job.plans[16].describe()["variants"]
    else:
        tensor_sweep = os.environ.get("BQA_GB300_TC", "1") != "0"
    kind = "tensor" if tensor_sweep else "cuda-core"
    roofline = {"kernel": "bp sweep (" + ("tcx_half_kernel_d3c16" if tensor_sweep else "tiled_half_kernel<3,16>") +
                          " + bp_combine_kernel)", "bound": "tensor",
                "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "peak_source": f"{pk_kind} bf16 burst",
                "traffic": (SWEEP_DRAM_BYTES_PER_NODE[kind] * n_el if args.chi == 16 else None),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 10k-node sweep "
                                  f"(half-node kernel {SWEEP_DRAM_BYTES_PER_NODE[kind] * 1e4 / 1e6 - 224.94:.1f} MB "
                                  "+ combine 224.9 MB), scaled by node count",
                "algorithmic_bytes_per_launch": bp_bytes / max(len(sweep_ev), 1),
                "algorithmic_flops_per_launch": bp_flops / max(len(sweep_ev), 1),
                "legacy_mma_peaks_measured": {"bf16_m16n8k16": mma_peak_tflops(dev, 0),
                                              "tf32_m16n8k8": mma_peak_tflops(dev, 1),
                                              "unit": "TFLOP/s", "probe": "bqa_mma_probe"}}
    if tensor_sweep and args.chi == 16:
        executed = achieved * TC_EXECUTED_FLOPS_PER_NODE / (16 * 9 * 16 ** 4)
        roofline["note"] = ("complex64 contraction on the tensor cores in 2xFP16 (every operand split into two "
                            "FP16 terms, FP32 accumulation): 16 d^2 chi^(d+1) FLOP per node per sweep in the "
                            "reference order; the tensor cores execute 2.33x that (3 product terms, 4 closing "
                            "terms, K-split closing stages); FP16 and BF16 dense rates are the same")
        roofline["tensor_executed"] = {"tflops": executed, "frac": executed / pk["bf16_tflops"],
                                       "flops_per_node": TC_EXECUTED_FLOPS_PER_NODE}
    else:
        roofline["note"] = ("complex64 SIMT contraction: 16 d^2 chi^(d+1) FLOP per node per sweep (reference "
                            "order; the kernel executes 54% of them at degree 3, chi 16); the FP32 CUDA-core "
                            "peak, measured below, is the ceiling of this kernel")
        roofline["fp32_simt"] = {"peak_measured": fp32_peak, "unit": "TFLOP/s",
                                 "achieved_executed": achieved * EXECUTED_FRACTION.get(args.chi, 1.0),
                                 "frac": achieved * EXECUTED_FRACTION.get(args.chi, 1.0) / fp32_peak,
                                 "probe": "bqa_fp32_fma_probe, 16 independent FMA chains per thread"}
    secondary = None
    if args.secondary:
        del job
        torch.cuda.empty_cache()
        mx = mixed_measurement(50000, 4, 3, 2, True)
        sw = sweep_measurement(2000, 4, 32, "single", "default", 3, 1)
        c1 = c1_job_measurement(not args.no_cpu_baseline)
        secondary = {
            "c1_job": c1,
            "mixed_degree_chi4": {"what": "300x300 periodic grid + 50,000 nodes of degree 2/3/5/6 (140k nodes), bond "
                                          "dim 4, saturated steps, autotuned, device-timed",
                                  "steps_per_s": mx["steps_per_s"], "ms_per_step_split": mx["ms_per_step_split"],
                                  "sweeps_per_step": mx["sweeps_per_step"]},
            "degree4_chi32_sweep": {"what": "one BP sweep, random 4-regular 2,000 nodes, bond dim 32 (16 MB node "
                                            "tensors, global-memory kernels), random Hermitian messages",
                                    "ms_per_sweep": sw["ms_per_sweep"], "tflops_algorithmic": sw["tflops"]}}
    if mixed is not None:
        mms = mixed.pop("ms_raw")
        mixed = {"value": replica_value(world, args.steps, mms), "unit": "steps/s", "ms_per_step": mms / args.steps,
                 "vs_plain": t_max / mms, **mixed, "accuracy": measured_accuracy(mixed=True),
                 "what": "Annealer(mixed=True): at bond dim 16 the degree-3 sweeps run the mixed kernel "
                         "(BF16 tensor-core products and closing contractions while the last BP distance is "
                         "above 2^-5, FP32-accurate 2xFP16 tensor-core sweeps after that), same schedule window, "
                         "device-timed"}
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD.format(n=args.n, chi=args.chi),
                   "window": f"steps {prep_steps + args.warmup}..{prep_steps + args.warmup + args.steps - 1} "
                             f"of 200 (bond dim saturated at step {prep_steps})",
                   "l2": "state (6.6 GB tensors + 0.6 GB messages) >> 129 MB L2; no flush needed",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "bp_msg_updates_per_s": ctx.edges_number * sum(sweeps) / (bp_ms / 1000.0) if bp_ms else None,
        "sweeps_per_step": float(np.mean(sweeps)), "bond_dim": window[-1]["bond_dim"],
        "time_split_ms": {k: round(v, 2) for k, v in sorted(by_name.items(), key=lambda kv: -kv[1])},
        "roofline": roofline,
        "e2e": {"value": replica_value(world, args.steps, 1000.0 * e2e_s), "unit": "steps/s", "h2d_bytes_per_step": 16,
                "d2h_bytes_per_step": int(n_el * 4 * 8 + 2 * args.chi * 4 + 64),
                "what": "Annealer.run_layer + bloch_vectors per step (host scalars in, all marginals out), "
                        "the timed window's steps replayed from a snapshot of its starting state"},
        "accuracy": accuracy,
        "mixed_precision": mixed,
        "serving": serving,
        "secondary": secondary,
        "autotune": tuned,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "prep": {"steps": prep_steps, "seconds": round(prep_s, 1)},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_sweep_mode(args) -> None:
    """Time the dominant kernel alone: one BP sweep over all nodes at a fixed bond dim, on
    random normalised node tensors with random Hermitian positive-definite trace-normalised
    messages (not diagonal: diagonal incoming messages take the kernels' bond-scaling path,
    which only the first sweep after a truncation sees).  Prints one JSON line."""
    print(json.dumps(sweep_measurement(args.n, args.degree, args.chi, args.precision, args.variant, args.steps,
                                       args.warmup)))


def c1_job_measurement(with_cpu: bool) -> dict:
    """The CPU-runnable configuration end to end: the 1000-qubit chi-4 job (random 3-regular,
    J, h ~ N(0,1), 100 steps, bp_eps 1e-6) from config to result list through
    bqa_gb300.run_qa (median of 3 after one untimed run), and through the oracle port of the
    reference algorithm (complex128, one run on the host cores)."""
    import logging as _logging
    import torch
    import bqa_gb300
    from bqa_gb300 import instances
    conf = instances.headline_cpu_job()
    bqa_gb300.run_qa(dict(conf))
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        bqa_gb300.run_qa(dict(conf))
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    out = {"what": "1000-qubit random 3-regular job, chi 4, 100 steps, config to result list",
           "gpu_run_qa_s": float(np.median(ts))}
    if with_cpu:
        from oracle import bqa_oracle as orc
        level = _logging.getLogger("oracle.bqa_oracle").level
        _logging.getLogger("oracle.bqa_oracle").setLevel(_logging.ERROR)
        t0 = time.perf_counter()
        orc.run_qa(dict(conf))
        out["cpu_reference_port_s"] = time.perf_counter() - t0
        _logging.getLogger("oracle.bqa_oracle").setLevel(level)
        out["cpu_cores"] = len(os.sched_getaffinity(0))
    return out


def sweep_measurement(n: int, degree: int, chi: int, precision: str = "single", variant_name: str = "default",
                      steps: int = 3, warmup: int = 1) -> dict:
    """run_sweep_mode's measurement: mean CUDA-event time of `steps` sweeps after `warmup`."""
    import torch
    from bqa_gb300 import instances
    from bqa_gb300.engine import Annealer, _ptr
    from bqa_gb300.layout import build_context
    conf = instances.headline_gpu_job(n=n, seed=0, chi=chi, degree=degree)
    ctx = build_context(conf)
    job = Annealer(ctx, precision=precision)
    gen = torch.Generator(device="cuda").manual_seed(0)
    for c in job.classes:
        size = c.count * 2 * chi ** c.degree
        t = torch.randn(size, dtype=job.msgs[0].dtype, device="cuda", generator=gen).view(c.count, -1)
        c.tensors[0][:size].copy_((t / t.norm(dim=1, keepdim=True)).view(-1))
    E = ctx.edges_number
    eye = torch.eye(chi, dtype=job.msgs[0].dtype, device="cuda")
    for e0 in range(0, E, 65536):
        e1 = min(E, e0 + 65536)
        x = torch.randn(e1 - e0, chi, chi, dtype=job.msgs[0].dtype, device="cuda", generator=gen)
        m = x @ x.conj().transpose(1, 2) + 0.1 * eye
        m = m / torch.diagonal(m, dim1=1, dim2=2).sum(-1).view(-1, 1, 1)
        job.msgs[0][e0 * chi * chi: e1 * chi * chi].copy_(m.reshape(-1))
    job.chi = job.chis = chi
    job.tcur = job.mcur = 0
    cls = job._class_array()
    flops, nbytes = job.bp_sweep_cost()

    variant = {"default": None, "tiled": 1, "generic": 2, "tensor": 3, "tensor-bf16": 4, "mixed": 5}[variant_name]
    plan = None if variant is None else (ctypes.c_int32 * len(job.classes))(*([variant] * len(job.classes)))

    def sweep():
        if plan is not None:
            job.lib.call("bqa_bp_sweep_plan", cls, len(job.classes), chi, job.dtype, plan, _ptr(job.msgs[0]),
                         _ptr(job.msgs[1]), _ptr(job.lu) if job.split_sweeps else None, ctx.edges_number,
                         _ptr(job.dist_parts), None, job.stream)
        elif job.split_sweeps:
            job.lib.call("bqa_bp_sweep_split", cls, len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                         _ptr(job.msgs[1]), _ptr(job.lu), ctx.edges_number, _ptr(job.dist_parts), None, job.stream)
        else:
            job.lib.call("bqa_bp_sweep", cls, len(job.classes), chi, job.dtype, _ptr(job.msgs[0]), _ptr(job.msgs[1]),
                         _ptr(job.dist_parts), None, job.stream)

    for _ in range(warmup):
        sweep()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in evs:
        a.record()
        sweep()
        b.record()
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    mean = float(np.mean(ms))
    del job
    torch.cuda.empty_cache()
    return {"mode": "sweep", "n": n, "degree": degree, "chi": chi, "precision": precision, "variant": variant_name,
            "sweeps": steps, "ms_per_sweep": mean, "ms_min": float(np.min(ms)),
            "tflops": flops / (mean / 1000) / 1e12, "algorithmic_gbs": nbytes / (mean / 1000) / 1e9,
            "algorithmic_flops_per_launch": flops, "algorithmic_bytes_per_launch": nbytes,
            "msg_updates_per_s": ctx.edges_number / (mean / 1000)}


def run_svd_mode(args) -> None:
    """Time the truncation factorisation alone (environment SVDs + bond canonicalisation) on the
    extended messages of a real saturated-regime state: the anneal runs untimed until the bond
    dim saturates, then K repetitions of the two Jacobi kernels are timed with CUDA events."""
    import torch
    from bqa_gb300 import instances
    from bqa_gb300.engine import Annealer, _ptr
    from bqa_gb300.layout import build_context
    ctx = build_context(instances.headline_gpu_job(n=args.n, seed=0, chi=args.chi))
    steps = [i for i in ctx.instructions if isinstance(i, dict)]
    job = Annealer(ctx, precision=args.precision)
    s = 0
    lib, st, E = job.lib, job.stream, ctx.edges_number
    if args.synthetic:
        # random Hermitian PSD 2chi x 2chi matrices with a graded spectrum (no anneal)
        chi = args.chi
        n = 2 * chi
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn(E, n, n, dtype=job.ext.dtype, device="cuda", generator=g)
        x = x * torch.logspace(0, -4, n, device="cuda").to(x.dtype)
        m = x @ x.conj().transpose(1, 2)
        m = m / torch.diagonal(m, dim1=1, dim2=2).sum(-1).view(E, 1, 1)
        job.ext[: E * n * n].copy_(m.reshape(-1))
        job.chi = job.chis = chi
    else:
        while job.bond_dim < args.chi and s < len(steps) - 1:
            job.run_layer(steps[s]["xtime"], steps[s]["ztime"])
            s += 1
        chi = job.chis
        n = 2 * chi
        lib.call("bqa_ext_msgs", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job._msgs_cur()),
                 _ptr(job.ext), float(steps[s]["ztime"]), st)
    ext = job.ext.clone()
    canon = torch.empty_like(job.ext)
    eps = float(ctx.pinv_eps)

    def env():
        lib.call("bqa_env_factor", _ptr(ext), E, n, job.dtype, eps, _ptr(job.lu), _ptr(job.ul), _ptr(job.status), st)

    def can():
        lib.call("bqa_bond_canon", _ptr(job.lu), _ptr(job.ul), E, n, job.dtype, eps, _ptr(canon), _ptr(job.lmbds),
                 _ptr(job.colmax), _ptr(job.status), st)

    out = {"mode": "svd", "n": args.n, "chi": chi, "matrices": E, "size": n, "step": s}
    for name, fn in (("env_factor", env), ("bond_canon", can)):
        for _ in range(args.warmup):
            fn()
        # profilers select the saturated-state launches by this range (--nvtx-include svd_timed/)
        torch.cuda.nvtx.range_push("svd_timed")
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in evs:
            a.record()
            fn()
            b.record()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out[name + "_ms"] = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    out["status"] = int(job.status.item())
    print(json.dumps(out))


def serving_stream(jobs: int, rate: float, seed: int = 0, wide: bool = False):
    """Poisson stream of annealing jobs (arrival time, config): random d-regular graphs with
    n log-uniform in [100, 20000], J = +-1, h ~ N(0, 0.5), 20 or 50 steps over T = steps / 10;
    d in {3, 4} and bond dim in {4, 8}, or (wide) d in {3, 4, 5} and bond dim in {4, 8, 16} with
    n capped at 4,000 for bond dim 16 and degree 5 kept at bond dims 4 and 8."""
    from bqa_gb300 import instances
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(jobs):
        t += rng.exponential(1.0 / rate)
        n = int(np.exp(rng.uniform(np.log(100), np.log(20000))))
        d = int(rng.choice([3, 4, 5] if wide else [3, 4]))
        chi = int(rng.choice(([4, 8] if d == 5 else [4, 8, 16]) if wide else [4, 8]))
        if chi == 16:
            n = min(n, 4000)
        n += (n * d) % 2
        steps = int(rng.choice([20, 50]))
        e = instances.random_regular_edges(n, d, seed * 100003 + k)
        conf = instances.qubo_config(e, 2.0 * rng.integers(0, 2, len(e)) - 1, rng.normal(0, 0.5, n),
                                     max_bond_dim=chi, bp_eps=1e-5, pinv_eps=1e-6, max_bp_iter_number=50,
                                     schedule=instances.anneal_schedule(steps / 10.0, steps))
        out.append((t, conf))
    return out


SERVING_STREAM = "random d-regular, d in {3,4}, n log-uniform in [100, 20000], chi in {4, 8}, 20 or 50 steps"
SERVING_STREAM_WIDE = ("random d-regular, d in {3,4,5}, n log-uniform in [100, 20000] (at most 4,000 at chi 16), "
                       "chi in {4, 8, 16} (4 or 8 at degree 5), 20 or 50 steps")


def serving_measurement(jobs: int, rate: float, seed: int = 1, wide: bool = False) -> dict:
    """p50/p99 job latency and jobs/s of one Poisson job stream through the continuous-batching
    server with packed BP runs (the jobs waiting for BP swept in shared launches), through the
    server with each job's BP run in its own launches, and with the same jobs run one at a time
    in arrival order (each job's latency then includes its wait behind the earlier ones).  All
    three start from configs already compiled into contexts, so all time device state set-up,
    the anneal and the read-out."""
    import torch
    import bqa_gb300
    from bqa_gb300 import config as cfg
    from bqa_gb300.engine import Annealer
    from bqa_gb300.layout import build_context
    from bqa_gb300.serve import JobServer

    def run_one(ctx):
        job = Annealer(ctx)
        out = []
        for ins in ctx.instructions:
            if isinstance(ins, dict):
                job.run_layer(ins["xtime"], ins["ztime"])
            elif ins == cfg.MEASURE:
                out.append(job.measure())
            else:
                out.append(job.bloch_vectors())
        torch.cuda.synchronize()
        return out

    stream = serving_stream(jobs, rate, seed=seed, wide=wide)
    bqa_gb300.run_qa(dict(stream[0][1]))              # warm-up: compile paths and allocator
    torch.cuda.synchronize()

    def serve(pack_bp: bool) -> dict:
        srv = JobServer(pack_bp=pack_bp)
        for t, conf in stream:
            srv.submit(dict(conf), arrival=t)
        srv._t0 = time.perf_counter()
        srv.run(timeout=1800)
        out = srv.stats()
        srv.close()
        return out

    serve(True)                                       # warm-up of the packed kernels
    served = serve(True)
    unpacked = serve(False)
    ctxs = [(t, build_context(dict(conf))) for t, conf in stream]
    t0 = time.perf_counter()
    lat = []
    for t, ctx in ctxs:
        now = time.perf_counter() - t0
        if now < t:
            time.sleep(t - now)
        run_one(ctx)
        lat.append(time.perf_counter() - t0 - t)
    seq_span = time.perf_counter() - t0 - ctxs[0][0]
    return {"rate_per_s": rate, "jobs": jobs, "served": served, "served_unpacked_bp": unpacked,
            "one_at_a_time": {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                              "jobs_per_s": jobs / seq_span}}


def run_serve_mode(args) -> None:
    """serving_measurement for every rate in --rates (or --rate)."""
    rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
    wide = args.serve_stream == "wide"
    results = [serving_measurement(args.jobs, rate, wide=wide) for rate in rates]
    print(json.dumps({"mode": "serve", "jobs": args.jobs, "stream": SERVING_STREAM_WIDE if wide else SERVING_STREAM,
                      "rates": results}))


def run_layout_mode(args) -> None:
    """Degree-class compilation of an n-node random 3-regular job: config analysis, host
    compiler and device compiler (kernels alone by CUDA events, and with the edge upload and
    map read-back), median of --steps runs after --warmup."""
    import torch
    from bqa_gb300 import config as cfg, instances, layout
    conf = instances.headline_gpu_job(n=args.n, steps=3)
    c = cfg.analyse_config(conf, edge_arrays=True)
    edges = c[cfg.EDGES_KEY].edges
    n = args.n

    def timed(fn):
        ts = []
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            if i >= args.warmup:
                ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3

    host_ms = timed(lambda: layout.compile_layout(edges, n))
    dev_ms = timed(lambda: layout.compile_layout_device(edges, n))
    ctx_ms = timed(lambda: layout.build_context(conf, layout_device="cuda"))
    # kernels alone: edges already on the device
    from bqa_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda")
    E = edges.shape[0]
    d_edges = torch.as_tensor(edges.astype(np.int32), device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    bufs = [torch.empty(n, **i32) for _ in range(5)]
    order = torch.empty(E, **i32)
    first, count, status = torch.empty(256, **i32), torch.empty(256, **i32), torch.zeros(1, **i32)
    node_ids, slots = torch.empty(n, **i32), torch.empty(3 * n, **i32)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ks = []
    for i in range(args.warmup + args.steps):
        e0.record(st)
        lib.call("bqa_layout_degrees", d_edges.data_ptr(), E, n, 255, bufs[0].data_ptr(), bufs[1].data_ptr(),
                 order.data_ptr(), bufs[2].data_ptr(), first.data_ptr(), count.data_ptr(), status.data_ptr(),
                 st.cuda_stream)
        lib.call("bqa_layout_class", 3, n, bufs[0].data_ptr(), bufs[1].data_ptr(), order.data_ptr(), n, E, None,
                 None, node_ids.data_ptr(), bufs[3].data_ptr(), None, slots.data_ptr(), None, None, None,
                 st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        if i >= args.warmup:
            ks.append(e0.elapsed_time(e1))
    print(json.dumps({"mode": "layout", "n": n, "directed_edges": int(E),
                      "host_compile_ms": host_ms, "device_compile_ms": dev_ms,
                      "device_kernels_ms": float(np.median(ks)),
                      "build_context_ms": ctx_ms}))


def run_small_mode(args) -> None:
    """The 1000-qubit chi-4 job (random 3-regular, J, h ~ N(0,1), T 10, 100 steps, bp_eps 1e-6,
    <= 100 sweeps) through run_qa, wall-clock from config to result after one untimed run,
    and the per-step time split (host overhead = wall minus device kernel time)."""
    import torch
    import bqa_gb300
    from bqa_gb300 import instances
    from bqa_gb300.engine import Annealer
    from bqa_gb300.layout import build_context
    conf = instances.headline_cpu_job()
    bqa_gb300.run_qa(dict(conf))
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        bqa_gb300.run_qa(dict(conf))
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    ctx = build_context(dict(conf))
    job = Annealer(ctx)
    job.enable_kernel_timing(True)
    steps = [i for i in ctx.instructions if isinstance(i, dict)]
    t0 = time.perf_counter()
    for ins in steps:
        job.run_layer(ins["xtime"], ins["ztime"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    kt = job.kernel_times()
    dev_ms = sum(k[1] for k in kt)
    print(json.dumps({"mode": "small", "job": "random 3-regular n=1000, chi 4, 100 steps",
                      "run_qa_s": float(np.median(ts)), "steps_per_s": len(steps) / float(np.median(ts)),
                      "steps_wall_s": wall, "device_kernel_s": dev_ms / 1e3,
                      "mean_sweeps": float(np.mean([w["sweeps"] for w in job.stats]))}))


def run_mixed_mode(args) -> None:
    """Mixed degrees (periodic grid, degree 4, plus a configuration-model graph with degrees in
    {2, 3, 5, 6}) at bond dim --chi: anneal until the bond dim saturates (at most 60 steps),
    then time --steps steps; per-kernel split by CUDA events.  --n sets the extra nodes and the
    grid side (sqrt(1.8 n)), the full mixed configuration being n = 50,000 (300 x 300)."""
    print(json.dumps(mixed_measurement(args.n, args.chi, args.steps, args.warmup, bool(args.autotune))))


def mixed_measurement(n: int, chi: int, n_steps: int, warmup: int, autotune: bool) -> dict:
    """run_mixed_mode's measurement."""
    import torch
    from bqa_gb300 import instances
    from bqa_gb300.engine import Annealer
    from bqa_gb300.layout import build_context
    side = max(4, int(round(np.sqrt(1.8 * n))))
    ctx = build_context(instances.mixed_degree_job(rows=side, cols=side, extra=n, chi=chi))
    steps = [i for i in ctx.instructions if isinstance(i, dict)]
    job = Annealer(ctx, autotune=autotune)
    s, t0 = 0, time.perf_counter()
    while job.bond_dim < chi and s < 60:
        job.run_layer(steps[s]["xtime"], steps[s]["ztime"])
        s += 1
    prep = time.perf_counter() - t0
    for i in range(warmup):
        job.run_layer(steps[s]["xtime"], steps[s]["ztime"])
        s += 1
    job.enable_kernel_timing(True)
    job.stats.clear()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_steps")
    a.record()
    for i in range(n_steps):
        job.run_layer(steps[s + i]["xtime"], steps[s + i]["ztime"])
    b.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = a.elapsed_time(b)
    split: dict = {}
    for name, t, _, _ in job.kernel_times():
        split[name] = round(split.get(name, 0.0) + t / n_steps, 2)
    out = {"mode": "mixed", "nodes": ctx.nodes_number, "classes": {int(d): L.batch_size for d, L in
           ctx.degree_to_layout.items()}, "chi": job.bond_dim, "prep_steps": s - warmup,
           "prep_s": round(prep, 1), "steps_per_s": n_steps / (ms / 1e3),
           "sweeps_per_step": float(np.mean([w["sweeps"] for w in job.stats])),
           "ms_per_step_split": split, "scratch_bytes": job.scratch_elems * 8,
           "autotune": ([job.plans[c].describe() for c in sorted(job.plans)] if job.autotune else "off")}
    del job
    torch.cuda.empty_cache()
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--chi", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mixed", type=int, default=1, help="also time the mixed-precision form (1) or not (0)")
    ap.add_argument("--secondary", type=int, default=1,
                    help="also time the 1000-qubit chi-4 job (GPU and CPU), the mixed-degree chi-4 job and a "
                         "degree-4 chi-32 sweep (1) or not (0)")
    ap.add_argument("--serve-jobs", type=int, default=64,
                    help="jobs of the serving stream measured beside the anneal (0: none)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: BP message kernels chosen per (degree, bond dim) by the autotuner; 0: built-in choice")
    ap.add_argument("--mode", default="anneal", choices=["anneal", "sweep", "svd", "serve", "layout", "small", "mixed"])
    ap.add_argument("--jobs", type=int, default=32)
    ap.add_argument("--rate", type=float, default=200.0,
                    help="serving stream arrival rate (jobs/s); the default is the top of the stated 1-200 sweep")
    ap.add_argument("--rates", default="", help="serve mode: comma-separated arrival rates (jobs/s)")
    ap.add_argument("--serve-stream", default="small", choices=["small", "wide"],
                    help="serving job mix: degrees 3-4 at bond dims 4/8 (small) or degrees 3-5 at bond dims 4/8/16")
    ap.add_argument("--precision", default="single", choices=["single", "double"])
    ap.add_argument("--degree", type=int, default=3, help="sweep mode: degree of the random regular graph")
    ap.add_argument("--variant", default="default",
                    choices=["default", "tiled", "generic", "tensor", "tensor-bf16", "mixed"],
                    help="sweep mode: message kernel of every class (bqa_bp_sweep_plan)")
    ap.add_argument("--synthetic", action="store_true",
                    help="svd mode: random graded Hermitian PSD matrices instead of an annealed state")
    args = ap.parse_args()
    # every Annealer of this process (run_qa, the job server, the modes below) tunes its BP
    # message kernels unless --autotune 0
    os.environ["BQA_GB300_AUTOTUNE"] = "1" if args.autotune else "0"
    logging.basicConfig(level=logging.ERROR)
    logging.getLogger("bqa_gb300").setLevel(logging.ERROR)
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.mode == "sweep":
        run_sweep_mode(args)
    elif args.mode == "svd":
        run_svd_mode(args)
    elif args.mode == "serve":
        run_serve_mode(args)
    elif args.mode == "layout":
        run_layout_mode(args)
    elif args.mode == "small":
        run_small_mode(args)
    elif args.mode == "mixed":
        run_mixed_mode(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
