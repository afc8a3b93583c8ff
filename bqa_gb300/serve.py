"""Continuous-batching job server: many annealing jobs resident on one GPU at once.

A job is a config dict (the reference DSL).  ``JobServer.submit`` queues it with its arrival
time; a dispatcher admits queued jobs in arrival order as soon as their HBM footprint fits
the budget next to the jobs already resident, so jobs that arrive while others run start
as memory frees up.  Each admitted job is driven by its own host thread on its own CUDA
stream: the library calls and device synchronisations release the interpreter lock, so
the kernels of concurrent jobs overlap on the device while every job keeps its own device
state (tensors, messages, scratch).  A job's footprint is released when it finishes.

Results are the ``run_qa`` result lists; ``stats()`` reports per-job latency (arrival to
result) percentiles and the throughput of the whole stream.  A job's result is the same
whether it runs alone or in a mix: the kernels are deterministic and jobs share no device
buffers.
"""
from __future__ import annotations

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
                 max_active: int = 64):
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
        return {"jobs": len(jobs), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "mean_s": float(lat.mean()), "jobs_per_s": len(jobs) / span if span > 0 else None,
                "steps": int(sum(sum(isinstance(i, dict) for i in j.ctx.instructions) for j in jobs)),
                "peak_active": self.peak_active, "peak_bytes": self.peak_bytes}
