"""Autotuner of the BP message kernels, per (degree, storage bond dim, precision, class size).

A BP sweep (reference ``_run_bp``, src/bqa/state.py:105-113 with ``Tensor.pass_msgs``,
src/bqa/backends.py:381-408) runs one message kernel per degree class.  Several kernels
compute the same messages (up to rounding), and which is fastest depends on the degree, the
bond dim and the number of nodes:

* the sweep's form: two-stage (every node writes its open-bond blocks P_0, P_1 to scratch,
  then one pass forms the messages) or one-stage (every node writes its messages);
* per class, within a form: the register-tiled kernel (half-node CTAs in the two-stage form,
  whole-node CTAs in the one-stage form; complex64, degree 2-4, bond dims 4/8/12/16), the
  generic shared-memory kernel (global-memory form for nodes beyond shared memory), or, in the
  two-stage form at degree 3, bond dim 16, the FP32-accurate tensor-core half-node kernel
  (tcgen05, bond products and closing contractions in 2xFP16; the library's default there);
* for the generic kernel, the warps per node (CTA size): its own choice (one thread per fibre,
  up to 8 warps, or up to 32 for nodes whose shared memory leaves room for at most two CTAs
  per SM) or 16 or 32 warps at bond dims <= 8.

``tune(annealer)`` times every candidate of every class on the job's live state (CUDA events
on the job's stream, a warm-up launch then ``reps`` timed launches, each reading the current
messages and writing the idle message buffer, so the job's state is untouched), keeps the
fastest per class and form, then times the two complete sweeps and keeps the faster form (on
the complex64 path the two-stage form unless the one-stage sweep is over 15% faster: a
converged two-stage run also hands the next step's extended messages their open-bond blocks).
Results are cached per process by (device, precision, degree, bond dim, class size rounded up
to a power of two), and optionally in a JSON file named by the environment variable
BQA_GB300_TUNE_CACHE, so a job pays for tuning only at (degree, bond dim) pairs no earlier job
of its size class has seen.  The engine applies a plan through ``bqa_job.sweep_variants``
(one row per bond dim) and ``bqa_bp_sweep_plan``.
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
from dataclasses import dataclass, field

from . import _lib

VARIANT_NAMES = {_lib.BQA_VARIANT_DEFAULT: "default", _lib.BQA_VARIANT_TILED: "tiled",
                 _lib.BQA_VARIANT_GENERIC: "generic", _lib.BQA_VARIANT_TENSOR: "tensor",
                 _lib.BQA_VARIANT_TENSOR_BF16: "tensor-bf16", _lib.BQA_VARIANT_MIXED: "mixed"}
_SPLIT = 1 << 20   # flag of a two-stage timing in the tuner's per-class records
SPLIT_BONUS = 1.15  # two-stage sweeps win unless one-stage ones are faster by more than 15%


def generic_warps(warps: int) -> int:
    """Plan entry of the generic kernel with CTAs of ``warps`` warps (bqa_bp_sweep_plan)."""
    return _lib.BQA_VARIANT_GENERIC | (int(warps) << 8)


def variant_name(v: int) -> str:
    """``generic/16w`` for the generic kernel at 16 warps per node, else the variant's name."""
    base = VARIANT_NAMES[v & 0xff]
    return f"{base}/{v >> 8}w" if v >> 8 else base

_LOCK = threading.Lock()
_CLASS_CACHE: dict[tuple, dict] = {}     # class key -> {"best": variant, "ms": {variant: ms}}
_FORM_CACHE: dict[tuple, dict] = {}      # job key -> {"split": bool, "ms": {"split": ms, "whole": ms}}
_LOADED = False


@dataclass
class Plan:
    """What the tuner chose for one job at one storage bond dim."""
    chis: int
    split: bool                                   # two-stage sweeps
    variants: list[int]                           # per engine class
    class_ms: list[dict] = field(default_factory=list)
    form_ms: dict = field(default_factory=dict)

    def describe(self) -> dict:
        return {"chi": self.chis, "form": "two-stage" if self.split else "one-stage",
                "variants": [variant_name(v) for v in self.variants],
                "class_ms": [{variant_name(int(k)): round(v, 4) for k, v in m.items()} for m in self.class_ms],
                "form_ms": {k: (round(v, 4) if v is not None else None) for k, v in self.form_ms.items()}}


def _tuplify(x):
    return tuple(_tuplify(y) for y in x) if isinstance(x, (list, tuple)) else x


def _bucket(count: int) -> int:
    return 1 << max(0, int(count - 1).bit_length())


def _cache_path() -> str | None:
    return os.environ.get("BQA_GB300_TUNE_CACHE") or None


def _load() -> None:
    global _LOADED
    if _LOADED:
        return
    _LOADED = True
    path = _cache_path()
    if not path or not os.path.exists(path):
        return
    try:
        with open(path) as f:
            data = json.load(f)
        for k, v in data.get("classes", []):
            _CLASS_CACHE[_tuplify(k)] = {"best": int(v["best"]), "ms": {int(a): float(b) for a, b in v["ms"].items()}}
        for k, v in data.get("forms", []):
            _FORM_CACHE[_tuplify(k)] = {"split": bool(v["split"]), "ms": dict(v["ms"])}
    except (OSError, ValueError, KeyError, TypeError):
        pass   # a stale or foreign cache file is ignored, never fatal


def _save() -> None:
    path = _cache_path()
    if not path:
        return
    data = {"classes": [[k, {"best": v["best"], "ms": {str(a): b for a, b in v["ms"].items()}}]
                        for k, v in _CLASS_CACHE.items()],
            "forms": [[k, v] for k, v in _FORM_CACHE.items()]}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f)
    os.replace(tmp, path)


def clear_cache() -> None:
    """Forget every tuning result of this process (the JSON file is left as it is)."""
    with _LOCK:
        _CLASS_CACHE.clear()
        _FORM_CACHE.clear()
        _PLAN_CACHE.clear()


def _missing_variant(e: "_lib.BqaError") -> bool:
    """The library has no kernel of this variant for the class (not a candidate); any other
    failure is an error."""
    return e.status == _lib.BQA_ERR_UNSUPPORTED


class _Timer:
    """Times launches of one job's sweeps with CUDA events on the job's stream."""

    def __init__(self, job, reps: int):
        self.job = job
        self.reps = max(1, int(reps))
        torch = job.torch
        self.dist = torch.zeros(2, dtype=torch.int64, device=job.device)

    def sweep(self, classes, variants, split: bool) -> None:
        job = self.job
        arr = (ctypes.c_int32 * len(variants))(*variants)
        job.lib.call("bqa_bp_sweep_plan", classes, len(variants), job.chis, job.dtype, arr,
                     job.msgs[job.mcur].data_ptr(), job.msgs[1 - job.mcur].data_ptr(),
                     job.lu.data_ptr() if split else None, job.E, self.dist.data_ptr(), None, job.stream)

    def time(self, classes, variants, split: bool, best: float | None = None) -> float | None:
        """Mean milliseconds of one sweep, or None when a variant does not exist for a class.  A
        candidate whose warm-up launch already takes over 4x ``best`` is not timed further (its
        warm-up time is returned)."""
        torch = self.job.torch
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        try:
            self.sweep(classes, variants, split)       # warm-up (also opts kernels into shared memory)
        except _lib.BqaError as e:
            if _missing_variant(e):
                return None
            raise
        ev1.record()
        ev1.synchronize()
        warm = ev0.elapsed_time(ev1)
        if best is not None and warm > 4.0 * best:
            return warm
        ev0.record()
        for _ in range(self.reps):
            self.sweep(classes, variants, split)
        ev1.record()
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / self.reps


_DEVICE_NAMES: dict = {}
_PLAN_CACHE: dict[tuple, Plan] = {}      # job key -> finished plan (fast path for repeated jobs)


def _device_name(job) -> str:
    idx = job.device.index if job.device.index is not None else job.torch.cuda.current_device()
    name = _DEVICE_NAMES.get(idx)
    if name is None:
        name = _DEVICE_NAMES[idx] = job.torch.cuda.get_device_name(idx)
    return name


def tune(job, reps: int = 3) -> Plan:
    """Choose the sweep form and each class's message kernel for ``job`` at its current storage
    bond dim (``job.chis``), timing candidates on its live state.  The job's tensors, current
    messages and loop state are not modified."""
    with _LOCK:
        _load()
    dev = _device_name(job)
    chis = job.chis
    jkey = (dev, job.precision, chis, tuple((c.degree, _bucket(c.count)) for c in job.classes))
    with _LOCK:
        done = _PLAN_CACHE.get(jkey)
    if done is not None:
        return Plan(chis=chis, split=done.split, variants=list(done.variants), class_ms=done.class_ms,
                    form_ms=done.form_ms)
    torch = job.torch
    classes = job._class_array()
    active = [i for i, c in enumerate(job.classes) if c.degree > 0 and c.count > 0]
    timer = None
    best: dict[bool, list[int]] = {}
    class_ms: list[dict] = [dict() for _ in job.classes]
    with torch.cuda.device(job.device):
        for split in (True, False):
            picks = [_lib.BQA_VARIANT_DEFAULT] * len(job.classes)
            for i in active:
                c = job.classes[i]
                key = (dev, job.precision, c.degree, chis, _bucket(c.count), split)
                with _LOCK:
                    hit = _CLASS_CACHE.get(key)
                if hit is None:
                    timer = timer or _Timer(job, reps)
                    one = (_lib.BqaClass * 1)(classes[i])
                    ms = {}
                    cands = [_lib.BQA_VARIANT_TILED, _lib.BQA_VARIANT_GENERIC]
                    if split and job.precision == "single" and c.degree == 3 and chis == 16:
                        cands.insert(1, _lib.BQA_VARIANT_TENSOR)
                    if chis <= 8 and c.degree >= 4:
                        cands += [generic_warps(16), generic_warps(32)]
                    for v in cands:
                        t = timer.time(one, [v], split, min(ms.values()) if ms else None)
                        if t is not None:
                            ms[v] = t
                    hit = {"best": min(ms, key=ms.get) if ms else _lib.BQA_VARIANT_DEFAULT, "ms": ms}
                    with _LOCK:
                        _CLASS_CACHE[key] = hit
                picks[i] = hit["best"]
                class_ms[i].update({(v | _SPLIT if split else v): t for v, t in hit["ms"].items()})
            best[split] = picks
        with _LOCK:
            form = _FORM_CACHE.get(jkey)
        if form is None:
            timer = timer or _Timer(job, reps)
            ms = {"split": timer.time(classes, best[True], True), "whole": timer.time(classes, best[False], False)}
            inf = float("inf")
            # a two-stage run that converges leaves the open-bond blocks the next step's extended
            # messages start from (one combine pass instead of a sweep-like pass); on the
            # complex64 path that is worth about one sweep per step, so the two-stage form is kept
            # unless the one-stage sweep is faster by more than SPLIT_BONUS
            bonus = SPLIT_BONUS if job.split_sweeps and job.reuse_blocks else 1.0
            form = {"split": (ms["split"] or inf) <= bonus * (ms["whole"] or inf), "ms": ms}
            with _LOCK:
                _FORM_CACHE[jkey] = form
                _save()
    split = bool(form["split"])
    per_class = [{k & (_SPLIT - 1): v for k, v in m.items() if bool(k & _SPLIT) == split} for m in class_ms]
    plan = Plan(chis=chis, split=split, variants=best[split], class_ms=per_class, form_ms=dict(form["ms"]))
    with _LOCK:
        _PLAN_CACHE[jkey] = plan
    return plan
