"""ctypes binding of ``libbqa_gb300.so`` (the C ABI declared in ``include/bqa_gb300.h``).

There is no fallback: if the library was not built, loading raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int32, c_int64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libbqa_gb300.so"
ABI_VERSION = 13
BQA_C64 = 0
BQA_C128 = 1
BQA_VARIANT_DEFAULT, BQA_VARIANT_TILED, BQA_VARIANT_GENERIC, BQA_VARIANT_TENSOR = 0, 1, 2, 3
BQA_VARIANT_TENSOR_BF16, BQA_VARIANT_MIXED = 4, 5

BQA_OK = 0
BQA_STATUS_SVD_NOT_CONVERGED = 1
BQA_STATUS_LAYOUT_EDGE = 2
BQA_STATUS_LAYOUT_DEGREE = 4


class BqaClass(ctypes.Structure):
    """Mirror of ``struct bqa_class``."""
    _fields_ = [
        ("degree", c_int32),
        ("count", c_int32),
        ("node_ids", c_void_p),
        ("in_pos", c_void_p),
        ("out_pos", c_void_p),
        ("lmbd_pos", c_void_p),
        ("edge_ampl", c_void_p),
        ("node_ampl", c_void_p),
        ("tensor", c_void_p),
        ("tensor_out", c_void_p),
        ("scratch", c_void_p),
        ("scratch_elems", c_int64),
    ]


class BqaJob(ctypes.Structure):
    """Mirror of ``struct bqa_job``."""
    _fields_ = [
        ("dtype", c_int32), ("n_classes", c_int32), ("classes", POINTER(BqaClass)),
        ("edges", c_int32), ("max_bond_dim", c_int32), ("max_bp_iters", c_int32), ("bp_check_every", c_int32),
        ("pad_bonds", c_int32), ("split_sweeps", c_int32), ("colmax_elems", c_int32),
        ("chi", c_int32), ("chis", c_int32), ("lam_stride", c_int32), ("mcur", c_int32), ("tcur", c_int32),
        ("bp_eps", c_double), ("pinv_eps", c_double), ("damping", c_double),
        ("msgs", c_void_p * 2), ("ext", c_void_p), ("lu", c_void_p), ("ul", c_void_p), ("lmbds", c_void_p),
        ("colmax", c_void_p), ("dist_parts", c_void_p), ("loop_state", c_void_p), ("status", c_void_p),
        ("edge_j", c_void_p), ("sweep_variants", POINTER(c_int32)), ("blocks_valid", c_int32),
    ]


class BqaLayerInfo(ctypes.Structure):
    """Mirror of ``struct bqa_layer_info``."""
    _fields_ = [("bond_dim", c_int32), ("sweeps", c_int32), ("bp_exhausted", c_int32),
                ("svd_not_converged", c_int32), ("trunc_err", c_double), ("best_dist", c_double)]


# name -> (restype, argtypes); every exported symbol of the header
SIGNATURES = {
    "bqa_abi_version": (c_int32, []),
    "bqa_launch_count": (c_int64, []),
    "bqa_last_error": (ctypes.c_char_p, []),
    "bqa_max_bond_dim": (c_int32, [c_int32, c_int32]),
    "bqa_node_scratch_elems": (c_int64, [c_int32, c_int32, c_int32]),
    "bqa_bp_sweep": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p]),
    "bqa_bp_sweep_split": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                     c_int32, c_void_p, c_void_p, c_void_p]),
    "bqa_bp_sweep_plan": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, POINTER(c_int32), c_void_p,
                                    c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p]),
    "bqa_tc_faults": (c_int32, [POINTER(c_int32), c_int32, c_void_p]),
    "bqa_bp_finalize": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_double, c_double,
                                  c_int32, c_void_p]),
    "bqa_ext_msgs": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_double, c_void_p]),
    "bqa_ext_msgs_split": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int32,
                                     c_void_p, c_double, c_void_p, c_void_p]),
    "bqa_ext_combine": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_double, c_void_p, c_void_p]),
    "bqa_env_factor": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_double, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "bqa_bond_canon": (c_int32, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_double, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p]),
    "bqa_apply_update": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int32,
                                   c_double, c_double, c_void_p]),
    "bqa_msgs_from_lmbds": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p]),
    "bqa_densities": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "bqa_psplit": (c_int32, [POINTER(BqaClass), c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "bqa_edge_zz": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p]),
    "bqa_lmbds_truncate": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_int32, c_void_p]),
    "bqa_project_nodes": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p,
                                    c_void_p]),
    "bqa_canonicalize_noalloc": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_double, c_void_p, c_void_p,
                                           c_void_p, c_void_p, c_void_p]),
    "bqa_run_layer": (c_int32, [POINTER(BqaJob), c_double, c_double, POINTER(BqaLayerInfo), c_void_p]),
    "bqa_graph_cache_create": (c_int32, [POINTER(c_void_p)]),
    "bqa_graph_cache_destroy": (c_int32, [c_void_p]),
    "bqa_run_layer_graph": (c_int32, [POINTER(BqaJob), c_void_p, c_double, c_double, POINTER(BqaLayerInfo),
                                      c_void_p]),
    "bqa_run_bp_graph": (c_int32, [POINTER(BqaJob), c_void_p, POINTER(BqaLayerInfo), c_void_p]),
    "bqa_gate_layer": (c_int32, [POINTER(BqaJob), c_double, c_double, POINTER(BqaLayerInfo), c_void_p]),
    "bqa_bp_begin": (c_int32, [POINTER(BqaJob), c_void_p]),
    "bqa_bp_packed": (c_int32, [POINTER(POINTER(BqaJob)), c_int32, c_int32, c_void_p, POINTER(c_int32), c_void_p]),
    "bqa_bp_end": (c_int32, [POINTER(BqaJob), POINTER(c_int32), POINTER(BqaLayerInfo)]),
    "bqa_layout_degrees": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_void_p]),
    "bqa_layout_class": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]),
}


BQA_ERR_UNSUPPORTED = 2


class BqaError(RuntimeError):
    """A library call returned a non-zero status (``status``: BQA_ERR_*)."""

    def __init__(self, message: str, status: int | None = None):
        super().__init__(message)
        self.status = status


class Library:
    """Loaded library with checked calls: ``lib.call("bqa_x", ...)`` raises on a bad status."""

    def __init__(self, path: Path = LIB_PATH):
        if not path.exists():
            raise BqaError(f"{path} is missing: build the GB300 backend first "
                           "(python -m bqa_gb300.build, or __graft_entry__.build())")
        self.path = path
        self.dll = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(self.dll, name)
            fn.restype = res
            fn.argtypes = args
        v = self.dll.bqa_abi_version()
        if v != ABI_VERSION:
            raise BqaError(f"{path} has ABI version {v}, expected {ABI_VERSION}: rebuild it")

    def call(self, name: str, *args) -> None:
        rc = getattr(self.dll, name)(*args)
        if rc != BQA_OK:
            msg = self.dll.bqa_last_error().decode(errors="replace")
            raise BqaError(f"{name} failed with status {rc}: {msg}", status=int(rc))

    def max_bond_dim(self, degree: int, dtype: int = BQA_C64) -> int:
        return int(self.dll.bqa_max_bond_dim(degree, dtype))

    def tc_faults(self, stream=None, reset: bool = True) -> int:
        """CTAs of the tensor-core kernels whose wait for their MMAs ran out (0 when healthy)."""
        out = c_int32(0)
        self.call("bqa_tc_faults", ctypes.byref(out), 1 if reset else 0, stream)
        return int(out.value)


_LIB: Library | None = None


def load() -> Library:
    global _LIB
    if _LIB is None:
        _LIB = Library()
    return _LIB


PROBE_LIB_PATH = Path(__file__).resolve().parent / "libbqa_gb300_probes.so"
PROBE_SIGNATURES = {
    "bqa_fp32_fma_probe": (c_int32, [c_int32, c_int32, c_void_p, c_void_p]),
    "bqa_mma_probe": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p]),
}
_PROBES = None


def load_probes():
    """The measurement probes' library (include/bqa_gb300_probes.h), separate from the backend."""
    global _PROBES
    if _PROBES is None:
        if not PROBE_LIB_PATH.exists():
            raise BqaError(f"{PROBE_LIB_PATH} is missing: build it with python -m bqa_gb300.build")
        dll = ctypes.CDLL(str(PROBE_LIB_PATH))
        for name, (res, args) in PROBE_SIGNATURES.items():
            fn = getattr(dll, name)
            fn.restype = res
            fn.argtypes = args
        _PROBES = dll
    return _PROBES
