"""Continuous-batching job server: many annealing jobs resident on one GPU at once.

A job is a config dict (the reference DSL).  ``JobServer.submit`` queues it with its arrival
time; a dispatcher admits queued jobs in arrival order as soon as their HBM footprint fits
the budget next to the jobs already resident, so jobs that arrive while others run start
as memory frees up.  Each admitted job is driven by its own host thread on its own CUDA
stream: the library calls and device synchronisations release the interpreter lock, so
the kernels of concurrent jobs overlap on the device while every job keeps its own device
state (tensors, messages, scratch).  A job's footprint is released when it finishes.

BP runs are packed (``pack_bp=True``, the default): after its gate layer a job hands its BP
run to a ``BpPacker``, which sweeps the runs of all the jobs waiting at that moment in shared
launches -- each node kernel once per sweep for the degree classes of every job that uses it,
one combine and one decision kernel for all of them (bqa_bp_packed) -- takes each job out when
its own loop state says done and lets newly waiting jobs join between sweep groups.  Jobs are
packed only with jobs of about the same sweep cost (one packer, thread and stream per factor-4
band of a sweep's FLOPs), so a small job never waits on a large job's sweeps; the bands' packs
run concurrently.

Results are the ``run_qa`` result lists; ``stats()`` reports per-job latency (arrival to
result) percentiles and the throughput of the whole stream.  A job's result is the same
whether it runs alone or in a mix, packed or not: the kernels are deterministic, a CTA
computes the same values in a shared launch as in the job's own, and jobs share no device
buffers.
"""
from __future__ import annotations

import ctypes
import heapq
import itertools
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from . import config as cfg
from .engine import Annealer, resolve_precision
from .layout import Context, build_context


def job_footprint(ctx: Context, precision: str | None = None, sm_count: int | None = None) -> int:
    """Device bytes an ``Annealer`` for ``ctx`` allocates (the buffers of its constructor).

    ``sm_count``: multiprocessors of the device the job runs on (the engine sizes the work
    tensors of classes beyond shared memory as 8 CTAs per SM); None asks the current CUDA
    device, or takes GB300's 152 where no GPU is visible (footprint planning on a host)."""
    p = resolve_precision(precision)
    es = 8 if p == "single" else 16
    rs = es // 2
    pad = p == "single" and all(d <= 4 for d in ctx.degree_to_layout)
    chi = ctx.max_bond_dim
    if pad and 4 < chi <= 16 and chi % 4:
        chi += 4 - chi % 4
    E, half, n = ctx.edges_number, ctx.edges_number // 2, ctx.nodes_number
    nmax = 2 * chi
    total = 0
    for d, L in ctx.degree_to_layout.items():
        B = L.batch_size
        total += 2 * B * 2 * chi ** d * es                 # tensors (ping-pong)
        total += B * (4 + 3 * 4 * d + 8 * d + 8)           # maps and amplitudes
    total += 2 * E * chi * chi * es                        # messages
    total += 3 * E * nmax * nmax * es                      # ext / lu / ul
    total += half * nmax * rs + n * 4 * es + half * 8      # lambdas, densities, <ZZ>
    # work tensors for classes beyond shared memory (engine: min(count, 8 x SMs) CTAs)
    if sm_count is None:
        import torch
        sm_count = (torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
                    if torch.cuda.is_available() else 152)
    lib = _lib.load()
    dt = _lib.BQA_C64 if p == "single" else _lib.BQA_C128
    total += max((min(L.batch_size, 8 * sm_count) * int(lib.dll.bqa_node_scratch_elems(d, chi, dt)) * es
                  for d, L in ctx.degree_to_layout.items()), default=0)
    return int(total) + (1 << 20)


class _BpRun:
    """One job's BP run handed to the packer."""

    def __init__(self, job, info):
        self.job = job            # the job's bqa_job struct (kept alive by the job's thread)
        self.info = info          # its bqa_layer_info, filled in by bqa_bp_end
        self.launched = 0
        self.error: BaseException | None = None
        self.done = threading.Event()


class BpPacker:
    """Sweeps the BP runs of the jobs waiting for one in shared launches (bqa_bp_packed).

    Job threads call ``run_bp`` after their gate layer (their stream synchronised) and block
    until their run is done.  One packer thread takes every waiting run (up to 64 at once),
    zeroes its loop state (bqa_bp_begin), launches ``sweeps_per_call`` packed sweeps, reads all
    loop states with one copy, and concludes the runs that are done (bqa_bp_end); runs that are
    not go on with the next sweep group, joined by runs that arrived meanwhile."""

    MAX_JOBS = 64

    def __init__(self, device=None, sweeps_per_call: int = 4):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        dev = torch.device(device if device is not None else "cuda")
        self.device = torch.device("cuda", dev.index if dev.index is not None else torch.cuda.current_device())
        self.sweeps_per_call = max(1, int(sweeps_per_call))
        self.stream = torch.cuda.Stream(device=self.device)
        self.ls_dev = torch.zeros(8 * self.MAX_JOBS, dtype=torch.int32, device=self.device)
        self.ls_host = (ctypes.c_int32 * (8 * self.MAX_JOBS))()
        self._cond = threading.Condition()
        self._waiting: list[_BpRun] = []
        self._stop = False
        self._died: BaseException | None = None
        self.calls = 0
        self.packed_runs = 0        # sum over calls of the runs swept together
        self.max_packed = 0
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    def run_bp(self, job, info) -> None:
        run = _BpRun(job, info)
        with self._cond:
            if self._stop or self._died is not None:
                raise RuntimeError("the BP packer is closed") from self._died
            self._waiting.append(run)
            self._cond.notify_all()
        while not run.done.wait(1.0):
            if not self._thread.is_alive():
                raise RuntimeError("the BP packer's thread ended") from self._died
        if run.error is not None:
            raise run.error

    def close(self) -> None:
        with self._cond:
            self._stop = True
            self._cond.notify_all()
        self._thread.join()

    def stats(self) -> dict:
        return {"packed_calls": self.calls, "sweeps_per_call": self.sweeps_per_call,
                "mean_runs_per_call": self.packed_runs / self.calls if self.calls else 0.0,
                "max_runs_per_call": self.max_packed}

    def _fail(self, runs, e: BaseException) -> None:
        for r in runs:
            r.error = e
            r.done.set()

    def _loop(self) -> None:
        active: list[_BpRun] = []
        try:
            self._serve(active)
        except BaseException as e:   # noqa: BLE001 -- every waiting job learns of it
            self._died = e
            with self._cond:
                waiting, self._waiting = self._waiting, []
            self._fail(active + waiting, e)

    def _serve(self, active: list) -> None:
        torch, lib = self.torch, self.lib
        torch.cuda.set_device(self.device)
        st = self.stream.cuda_stream
        while True:
            with self._cond:
                while not self._waiting and not active and not self._stop:
                    self._cond.wait()
                if self._stop and not active:
                    self._fail(self._waiting, RuntimeError("the BP packer is closed"))
                    self._waiting = []
                    return
                room = self.MAX_JOBS - len(active)
                new, self._waiting = self._waiting[:room], self._waiting[room:]
            for r in new:
                try:
                    lib.call("bqa_bp_begin", ctypes.byref(r.job), st)
                    active.append(r)
                except BaseException as e:   # noqa: BLE001 -- reported to the job's thread
                    self._fail([r], e)
            if not active:
                continue
            n = len(active)
            jobs = (ctypes.POINTER(_lib.BqaJob) * n)(*[ctypes.pointer(r.job) for r in active])
            try:
                lib.call("bqa_bp_packed", jobs, n, self.sweeps_per_call, self.ls_dev.data_ptr(), self.ls_host, st)
            except BaseException as e:   # noqa: BLE001
                self._fail(active, e)
                active.clear()
                continue
            self.calls += 1
            self.packed_runs += n
            self.max_packed = max(self.max_packed, n)
            still = []
            for i, r in enumerate(active):
                r.launched += self.sweeps_per_call
                ls = (ctypes.c_int32 * 8)(*self.ls_host[8 * i: 8 * i + 8])
                if ls[0]:
                    try:
                        lib.call("bqa_bp_end", ctypes.byref(r.job), ls, ctypes.byref(r.info))
                    except BaseException as e:   # noqa: BLE001
                        r.error = e
                    r.done.set()
                elif r.launched >= r.job.max_bp_iters + self.sweeps_per_call:
                    self._fail([r], RuntimeError("BP loop state did not finish after the iteration cap"))
                else:
                    still.append(r)
            active[:] = still


@dataclass(order=True)
class _Job:
    arrival: float
    seq: int
    config: dict = field(compare=False)
    ctx: Context = field(compare=False, default=None)
    footprint: int = field(compare=False, default=0)
    start: float = field(compare=False, default=0.0)
    end: float = field(compare=False, default=0.0)
    result: list = field(compare=False, default=None)
    error: BaseException = field(compare=False, default=None)


class JobServer:
    """Admit jobs by HBM footprint, run them concurrently, one stream and host thread each."""

    def __init__(self, hbm_budget: int | None = None, device=None, precision: str | None = None,
                 max_active: int = 64, pack_bp: bool = True):
        import torch
        self.torch = torch
        self.device = torch.device(device if device is not None else "cuda")
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(free * 0.85)
        self.budget = int(hbm_budget)
        self.sm_count = (torch.cuda.get_device_properties(self.device).multi_processor_count
                         if self.device.type == "cuda" else None)
        self.precision = precision
        self.max_active = max_active
        self._queue: list[_Job] = []
        self._seq = itertools.count()
        self._lock = threading.Condition()
        self._in_use = 0
        self._active = 0
        self._threads: list[threading.Thread] = []
        self.done: dict[int, _Job] = {}
        self.peak_active = 0
        self.peak_bytes = 0
        self._t0 = time.perf_counter()
        self.pack_bp = bool(pack_bp) and self.device.type == "cuda"
        self._packers: dict[int, BpPacker] = {}
        self._packers_lock = threading.Lock()

    # ---- submission --------------------------------------------------------------------
    def now(self) -> float:
        return time.perf_counter() - self._t0

    def submit(self, config: dict, arrival: float | None = None) -> int:
        """Queue a job (arrival = now by default); returns its id.  Configs that cannot fit the
        budget even alone are rejected with ValueError."""
        ctx = build_context(config, layout_device=self.device)
        fp = job_footprint(ctx, self.precision, self.sm_count)
        if fp > self.budget:
            raise ValueError(f"job needs {fp} device bytes, above the server budget {self.budget}")
        job = _Job(self.now() if arrival is None else arrival, next(self._seq), config, ctx, fp)
        with self._lock:
            heapq.heappush(self._queue, job)
            self._lock.notify_all()
        return job.seq

    # ---- execution ---------------------------------------------------------------------
    def _run_job(self, job: _Job) -> None:
        torch = self.torch
        try:
            stream = torch.cuda.Stream(device=self.device)
            with torch.cuda.device(self.device), torch.cuda.stream(stream):
                annealer = Annealer(job.ctx, device=self.device, precision=self.precision)
                out = []
                for ins in job.ctx.instructions:
                    if isinstance(ins, dict):
                        if self.pack_bp:
                            annealer.run_layer_packed(ins["xtime"], ins["ztime"], self.packer_for)
                        else:
                            annealer.run_layer(ins["xtime"], ins["ztime"])
                    elif ins == cfg.MEASURE:
                        out.append(["measurement_outcomes", annealer.measure()])
                    else:
                        out.append(["bloch_vectors", annealer.bloch_vectors().tolist()])
                stream.synchronize()
                del annealer
            job.result = out
        except BaseException as e:   # a failed job must release its admission
            job.error = e
        job.end = self.now()
        with self._lock:
            self._in_use -= job.footprint
            self._active -= 1
            self.done[job.seq] = job
            self._lock.notify_all()

    def run(self, expected: int | None = None, timeout: float | None = None) -> dict[int, list]:
        """Dispatch until the queue is empty and every admitted job finished (or ``expected``
        jobs are done); returns ``{job id: result}``.  Jobs whose arrival time lies in the
        future are admitted when that time comes."""
        deadline = None if timeout is None else time.perf_counter() + timeout
        while True:
            with self._lock:
                finished = expected is not None and len(self.done) >= expected
                if finished or (not self._queue and self._active == 0 and expected is None):
                    break
                if deadline is not None and time.perf_counter() > deadline:
                    raise TimeoutError("job server did not drain before the timeout")
                job = self._queue[0] if self._queue else None
                now = self.now()
                if job is not None and job.arrival <= now and self._active < self.max_active \
                        and self._in_use + job.footprint <= self.budget:
                    heapq.heappop(self._queue)
                    self._in_use += job.footprint
                    self._active += 1
                    self.peak_active = max(self.peak_active, self._active)
                    self.peak_bytes = max(self.peak_bytes, self._in_use)
                    job.start = now
                    t = threading.Thread(target=self._run_job, args=(job,), daemon=True)
                    self._threads.append(t)
                    t.start()
                    continue
                wait = 0.05 if job is None else max(0.0, min(0.05, job.arrival - now)) or 0.005
                self._lock.wait(timeout=wait)
        for t in self._threads:
            t.join()
        errors = [j for j in self.done.values() if j.error is not None]
        if errors:
            raise RuntimeError(f"{len(errors)} job(s) failed; first: {errors[0].error!r}") from errors[0].error
        return {k: j.result for k, j in self.done.items()}

    def stats(self) -> dict:
        jobs = list(self.done.values())
        if not jobs:
            return {}
        lat = np.array([j.end - j.arrival for j in jobs])
        span = max(j.end for j in jobs) - min(j.arrival for j in jobs)
        out = {"jobs": len(jobs), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
               "mean_s": float(lat.mean()), "jobs_per_s": len(jobs) / span if span > 0 else None,
               "steps": int(sum(sum(isinstance(i, dict) for i in j.ctx.instructions) for j in jobs)),
               "peak_active": self.peak_active, "peak_bytes": self.peak_bytes}
        if self._packers:
            per = {band: p.stats() for band, p in sorted(self._packers.items())}
            calls = sum(v["packed_calls"] for v in per.values())
            runs = sum(v["mean_runs_per_call"] * v["packed_calls"] for v in per.values())
            out["bp_packing"] = {"packed_calls": calls,
                                 "sweeps_per_call": next(iter(per.values()))["sweeps_per_call"],
                                 "mean_runs_per_call": runs / calls if calls else 0.0,
                                 "max_runs_per_call": max(v["max_runs_per_call"] for v in per.values()),
                                 "bands": len(per)}
        return out

    def close(self) -> None:
        """Stop the BP packers' threads (the server takes no jobs afterwards)."""
        with self._packers_lock:
            packers, self._packers = list(self._packers.values()), {}
        for p in packers:
            p.close()

    def packer_for(self, sweep_flops: float) -> "BpPacker":
        """The packer of the factor-4 band of a sweep's FLOPs (created on first use)."""
        band = int(np.log2(max(sweep_flops, 1.0)) // 2)
        with self._packers_lock:
            p = self._packers.get(band)
            if p is None:
                p = self._packers[band] = BpPacker(self.device)
            return p
