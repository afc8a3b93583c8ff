"""The GB300 backend inside the reference ``bqa`` package: a registry entry plus a dispatch of
bqa's own compiled context to the device engine.

The reference selects a backend by the config's ``"backend"`` string, looked up in
``bqa.backends.BACKEND_STR_TO_BACKEND`` (``src/bqa/backends.py:26``; validated in
``src/bqa/config/config_syntax.py:63-70``, used in
``src/bqa/config/config_canonicalization.py:211``).  Its numpy and CuPy backends implement the
per-operation ``Tensor`` ABC (``src/bqa/backends.py:28-251``) that the state VM
(``src/bqa/state.py``) drives one batched op at a time.  The GB300 backend fuses whole phases
of an annealing step into kernels, so it joins bqa at two points:

* ``"gb300"`` is registered as a real ``Tensor`` subclass (``GB300Backend``, made by
  ``register()`` from the installed bqa's own ABC).  Its constructors and getters build and
  return host numpy arrays, exactly what bqa's config compiler needs: ``config_to_context``
  (``src/bqa/config/core.py:8``) runs unchanged for a gb300 config and produces bqa's own
  ``Context`` -- the degree-class layouts, message/lambda slot maps, amplitudes and the
  instruction list.  The per-operation arithmetic methods raise ``NotImplementedError``: the
  fused engine replaces the state VM, not its single ops.
* ``bqa.run_qa`` / ``bqa.core.run_qa`` are wrapped so a config whose backend is ``"gb300"``
  goes through bqa's own ``config_to_context`` and then ``run_context``, which converts that
  context into the engine's layout and executes the instructions on the GPU (the part of
  ``src/bqa/core.py:13-35`` after ``config_to_context``).  Every other config goes to the
  original function unchanged.  Same config dict in, same result list out.
"""
from __future__ import annotations

import functools
import importlib
from types import SimpleNamespace

import numpy as np

BACKEND_NAME = "gb300"
_BACKEND_CLASS = None


def _fused_only(name):
    def op(*_, **__):
        raise NotImplementedError(
            f"Tensor.{name}: the gb300 backend runs whole annealing steps as fused GPU kernels; "
            "bqa.run_qa hands a gb300 context to bqa_gb300.plugin.run_context")
    op.__name__ = name
    return op


def make_backend_class(tensor_abc):
    """A ``Tensor`` subclass whose raw tensors are host numpy arrays (constructors, getters), with
    every per-operation method raising ``NotImplementedError``."""

    def __init__(self, arr):
        self._tensor = arr

    def make_from_list(cls, lst):
        # index maps stay integers (the reference's np.intp), amplitudes complex128
        # (src/bqa/backends.py:583-585)
        dtype = np.intp if lst and isinstance(lst[0], (int, np.integer)) else np.complex128
        return cls(np.array(lst, dtype=dtype))

    def make_from_numpy(cls, arr):
        return cls(arr)

    def make_from_raw_tensor(cls, raw):
        return cls(raw)

    def make_constant(cls, const):
        return cls(np.array(const))

    def make_empty_raw_tensor(batch_size, shape):
        return np.empty((batch_size, *shape), dtype=np.complex128)

    ns = {
        "__init__": __init__,
        "__doc__": "bqa backend 'gb300': host numpy raw tensors; annealing runs in bqa_gb300's fused engine.",
        "make_from_list": classmethod(make_from_list),
        "make_from_numpy": classmethod(make_from_numpy),
        "make_from_raw_tensor": classmethod(make_from_raw_tensor),
        "make_constant": classmethod(make_constant),
        "make_empty_raw_tensor": staticmethod(make_empty_raw_tensor),
        "raw_tensor": property(lambda self: self._tensor),
        "numpy": property(lambda self: np.asarray(self._tensor)),
        "raw_shape": property(lambda self: tuple(self._tensor.shape[1:])),
    }
    for name in getattr(tensor_abc, "__abstractmethods__", ()):
        if name not in ns:
            ns[name] = staticmethod(_fused_only(name))
    return type("GB300Backend", (tensor_abc,), ns)


def context_from_reference(ref_ctx):
    """The engine's ``layout.Context`` from bqa's ``Context`` (``config_canonicalization.py:143-167``):
    the layouts' index maps and amplitudes, the run parameters and the instruction list."""
    from .layout import Context, DegreeClass

    def arr(t):
        return np.asarray(t.numpy if hasattr(t, "numpy") else t)

    n, E = int(ref_ctx.nodes_number), int(ref_ctx.edges_number)
    half = E // 2
    layouts = {}
    for d, L in ref_ctx.degree_to_layout.items():
        d = int(d)
        node_ids = arr(L.node_ids).astype(np.int64)
        B = node_ids.shape[0]

        def stack(ts, dtype):
            return (np.stack([arr(t) for t in ts]).astype(dtype) if d > 0 else np.zeros((0, B), dtype=dtype))

        layouts[d] = DegreeClass(
            degree=d, node_ids=node_ids,
            input_msgs_position=stack(L.input_msgs_position, np.int64),
            output_msgs_position=stack(L.output_msgs_position, np.int64),
            lmbds_position=stack(L.lmbds_position, np.int64),
            node_ampls=np.real(arr(L.node_ampls)).astype(np.float64),
            edge_ampls=np.real(stack(L.edge_ampls, np.complex128)).astype(np.float64))
    node_degree = np.empty(n, dtype=np.int64)
    node_position = np.empty(n, dtype=np.int64)
    for v, (d, p) in ref_ctx.path_to_tensors.items():
        node_degree[int(v)], node_position[int(v)] = int(d), int(p)
    edge_src = np.empty(half, dtype=np.int64)
    edge_dst = np.empty(half, dtype=np.int64)
    edge_ampl = np.empty(half, dtype=np.float64)
    for (u, v), pos in ref_ctx.edge_to_msg_pos.items():
        if pos < half:
            edge_src[pos], edge_dst[pos] = int(u), int(v)
            edge_ampl[pos] = float(np.real(ref_ctx.edge_to_ampl[(u, v)]))
    node_ampl = np.array([float(np.real(ref_ctx.node_to_ampl[v])) for v in range(n)], dtype=np.float64)
    return Context(
        nodes_number=n, edges_number=E, max_bond_dim=int(ref_ctx.max_bond_dim),
        max_bp_iters_number=int(ref_ctx.max_bp_iters_number), bp_eps=float(ref_ctx.bp_eps),
        pinv_eps=float(ref_ctx.pinv_eps), measurement_threshold=float(ref_ctx.measurement_threshold),
        damping=float(ref_ctx.damping), seed=int(ref_ctx.seed), instructions=list(ref_ctx.instructions),
        degree_to_layout=layouts, node_degree=node_degree, node_position=node_position,
        edge_src=edge_src, edge_dst=edge_dst, edge_ampl=edge_ampl, node_ampl=node_ampl)


def run_context(ref_ctx, device=None, as_arrays: bool = False) -> list:
    """Execute a bqa ``Context`` compiled for the gb300 backend on the GPU; the result list of
    ``src/bqa/core.py:13-35``."""
    from .core import run_compiled
    return run_compiled(context_from_reference(ref_ctx), device=device, as_arrays=as_arrays)


def reference_like_context(arrays) -> SimpleNamespace:
    """A stand-in with the attributes of bqa's ``Context`` (``config_canonicalization.py:143-167``)
    rebuilt from the arrays ``tests/golden/make_plugin_context.py`` recorded off a context that
    bqa's own ``config_to_context`` built for a gb300 config (the GPU hosts cannot import bqa)."""
    layouts = {}
    for d in [int(x) for x in arrays["degrees"]]:
        def k(name, d=d):
            return arrays[f"d{d}_{name}"]
        layouts[d] = SimpleNamespace(
            node_ids=k("node_ids"), input_msgs_position=list(k("input_msgs_position")),
            output_msgs_position=list(k("output_msgs_position")), lmbds_position=list(k("lmbds_position")),
            node_ampls=k("node_ampls"), edge_ampls=list(k("edge_ampls")))
    p2t = {int(v): (int(d), int(p)) for v, d, p in arrays["path_to_tensors"]}
    keys = [(int(u), int(v)) for u, v, _ in arrays["edge_to_msg_pos"]]
    e2m = {key: int(p) for key, (_, _, p) in zip(keys, arrays["edge_to_msg_pos"])}
    e2a = {key: float(a) for key, a in zip(keys, arrays["edge_ampl_by_key"])}
    n2a = {int(v): float(a) for v, a in enumerate(arrays["node_ampl"])}
    instructions = []
    for kind, (xt, zt) in zip(arrays["ins_kind"], arrays["ins_times"]):
        kind = str(kind)
        instructions.append({"type": kind, "xtime": float(xt), "ztime": float(zt)} if kind.endswith("evolution")
                            else kind)
    f = {k: float(v) for k, v in zip(arrays["scalar_names"], arrays["scalar_values"])}
    return SimpleNamespace(
        nodes_number=int(f["nodes_number"]), edges_number=int(f["edges_number"]),
        max_bond_dim=int(f["max_bond_dim"]), max_bp_iters_number=int(f["max_bp_iters_number"]),
        bp_eps=f["bp_eps"], pinv_eps=f["pinv_eps"], measurement_threshold=f["measurement_threshold"],
        damping=f["damping"], seed=int(f["seed"]), instructions=instructions, degree_to_layout=layouts,
        path_to_tensors=p2t, edge_to_msg_pos=e2m, edge_to_ampl=e2a, node_to_ampl=n2a)


SCALARS = ("nodes_number", "edges_number", "max_bond_dim", "max_bp_iters_number", "bp_eps", "pinv_eps",
           "measurement_threshold", "damping", "seed")


def record_context(ref_ctx) -> dict:
    """Arrays (no Python objects) that ``reference_like_context`` rebuilds ``ref_ctx`` from."""
    out = {"degrees": np.array([int(d) for d in ref_ctx.degree_to_layout], dtype=np.int64)}   # dict order
    for d, L in ref_ctx.degree_to_layout.items():
        B = len(np.asarray(L.node_ids.numpy))

        def stack(ts, dtype):
            return (np.stack([np.asarray(t.numpy) for t in ts]).astype(dtype) if ts
                    else np.zeros((0, B), dtype=dtype))

        out[f"d{d}_node_ids"] = np.asarray(L.node_ids.numpy).astype(np.int64)
        out[f"d{d}_input_msgs_position"] = stack(L.input_msgs_position, np.int64)
        out[f"d{d}_output_msgs_position"] = stack(L.output_msgs_position, np.int64)
        out[f"d{d}_lmbds_position"] = stack(L.lmbds_position, np.int64)
        out[f"d{d}_node_ampls"] = np.asarray(L.node_ampls.numpy)
        out[f"d{d}_edge_ampls"] = stack(L.edge_ampls, np.complex128)
    out["path_to_tensors"] = np.array([(v, d, p) for v, (d, p) in ref_ctx.path_to_tensors.items()], dtype=np.int64)
    out["edge_to_msg_pos"] = np.array([(u, v, p) for (u, v), p in ref_ctx.edge_to_msg_pos.items()], dtype=np.int64)
    out["edge_ampl_by_key"] = np.array([float(np.real(ref_ctx.edge_to_ampl[k])) for k in ref_ctx.edge_to_msg_pos])
    out["node_ampl"] = np.array([float(np.real(ref_ctx.node_to_ampl[v])) for v in range(ref_ctx.nodes_number)])
    out["ins_kind"] = np.array([i["type"] if isinstance(i, dict) else i for i in ref_ctx.instructions])
    out["ins_times"] = np.array([(i["xtime"], i["ztime"]) if isinstance(i, dict) else (0.0, 0.0)
                                 for i in ref_ctx.instructions], dtype=np.float64).reshape(-1, 2)
    out["scalar_names"] = np.array(SCALARS)
    out["scalar_values"] = np.array([float(getattr(ref_ctx, k)) for k in SCALARS])
    return out


def _wrap(original, config_to_context):
    if getattr(original, "_bqa_gb300_wrapped", False):
        return original

    @functools.wraps(original)
    def run_qa(config, *args, **kwargs):
        if isinstance(config, dict) and config.get("backend") == BACKEND_NAME:
            return run_context(config_to_context(config))
        return original(config, *args, **kwargs)

    run_qa._bqa_gb300_wrapped = True
    return run_qa


def register() -> bool:
    """Install the backend into an importable ``bqa``; returns False if bqa is absent."""
    global _BACKEND_CLASS
    try:
        bqa = importlib.import_module("bqa")
        backends = importlib.import_module("bqa.backends")
        core = importlib.import_module("bqa.core")
        config_core = importlib.import_module("bqa.config.core")
    except ImportError:
        return False
    if _BACKEND_CLASS is None or not issubclass(_BACKEND_CLASS, backends.Tensor):
        _BACKEND_CLASS = make_backend_class(backends.Tensor)
    backends.BACKEND_STR_TO_BACKEND[BACKEND_NAME] = _BACKEND_CLASS
    core.run_qa = _wrap(core.run_qa, config_core.config_to_context)
    bqa.run_qa = _wrap(bqa.run_qa, config_core.config_to_context)
    return True
