"""Device-resident annealing state and the per-step driver (the reference's state VM).

``Annealer`` holds one job on one GPU: the degree-class index maps (int32), the node
tensors of every class, the BP messages and the bond spectra, all resident in HBM, plus
the scratch of the simple update.  Its methods mirror ``src/bqa/state.py``:

============================  ==========================================  =====================
reference (src/bqa/state.py)  here                                        C-ABI calls
============================  ==========================================  =====================
``_initialize_state`` :67     ``Annealer.__init__`` / ``reset``           msgs_from_lmbds
``_simple_update`` :230       ``gate_layer``                              ext_msgs, env_factor,
                                                                          bond_canon, apply_update
``_apply_z/x_layer`` :142-156 fused into ``gate_layer``                   apply_update
``_set_to_symmetric_gauge``   fused into ``gate_layer``                   apply_update, msgs_from_lmbds
``_run_bp`` :97               ``run_bp``                                  bp_sweep, bp_finalize
``run_layer`` :315            ``run_layer``
``get_density_matrices`` :77  ``density_matrices``                        densities
``measure`` :250              ``measure``                                 densities (+ host loop)
(none)                        ``edge_zz`` / ``energy``                    psplit, edge_zz
============================  ==========================================  =====================

PyTorch only allocates device memory and supplies the stream; all arithmetic runs in
``libbqa_gb300.so``.
"""
from __future__ import annotations

import ctypes

import logging
from dataclasses import dataclass

import numpy as np

from . import _lib
from .layout import Context

log = logging.getLogger(__name__)

INIT_STATE = (np.sqrt(0.5), -np.sqrt(0.5))   # src/bqa/state.py:21


def resolve_precision(precision: str | None = None) -> str:
    """Arithmetic of a job: "single" (complex64, this backend's default) or "double" (complex128).

    Without an explicit argument the reference's switch is honoured: the environment
    variable BQA_PRECISION (src/bqa/utils.py:10-21); unset means "single" here, because
    the FP32 path is this backend's production path."""
    import os
    p = (precision or os.environ.get("BQA_PRECISION") or "single").lower()
    if p not in ("single", "double"):
        raise ValueError(f"Unknown value of BQA_PRECISION environment variable {p}")
    return p


def _ptr(t) -> int:
    return t.data_ptr() if t is not None and t.numel() > 0 else 0


@dataclass
class _DeviceClass:
    degree: int
    count: int
    node_ids: object
    in_pos: object
    out_pos: object
    lmbd_pos: object
    edge_ampl: object
    node_ampl: object
    tensors: list          # two ping-pong buffers, flat complex


class Annealer:
    """One annealing job resident on one GPU."""

    def __init__(self, ctx: Context, device=None, precision: str | None = None, bp_check_every: int = 4,
                 pad_bonds: bool | None = None, native: bool = True, graphs: bool | None = None,
                 autotune: bool | None = None, reuse_blocks: bool | None = None, mixed: bool | None = None):
        import torch
        self.torch = torch
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 backend needs a CUDA device")
        self.lib = _lib.load()
        self.precision = resolve_precision(precision)
        self.dtype = _lib.BQA_C64 if self.precision == "single" else _lib.BQA_C128
        cplx = torch.complex64 if self.precision == "single" else torch.complex128
        real = torch.float32 if self.precision == "single" else torch.float64
        self.real_np = np.float32 if self.precision == "single" else np.float64
        self.ctx = ctx
        # steps through bqa_run_layer (one library call per step, no interpreter lock held);
        # per-kernel timing runs the same launches from Python
        self.native = bool(native)
        # BP runs replayed as captured CUDA graphs (one launch and one host read per run) unless
        # graphs=False or the environment variable BQA_GB300_GRAPHS=0
        if graphs is None:
            import os
            graphs = os.environ.get("BQA_GB300_GRAPHS", "1") != "0"
        self.graphs = bool(graphs)
        self._graph_cache = None
        # per-(degree, bond dim) choice of the BP message kernels (autotune.py) when autotune=True or
        # the environment variable BQA_GB300_AUTOTUNE=1; the plan of bond dim chis is row chis of
        # the table handed to the native driver (entry 0 the sweep form, then one entry per class)
        if autotune is None:
            import os
            autotune = os.environ.get("BQA_GB300_AUTOTUNE", "0") == "1"
        self.autotune = bool(autotune)
        self.plans: dict = {}
        # A BP run that converged with two-stage sweeps leaves in lu the open-bond blocks of the
        # messages it keeps (its last sweep's input); the next gate layer then forms the extended
        # messages from them with one combine pass (off with reuse_blocks=False or
        # BQA_GB300_REUSE_BLOCKS=0).  Anything that changes tensors, messages or lu clears it.
        if reuse_blocks is None:
            import os
            reuse_blocks = os.environ.get("BQA_GB300_REUSE_BLOCKS", "1") != "0"
        self.reuse_blocks = bool(reuse_blocks)
        self.blocks_valid = False
        self.device = torch.device(device if device is not None else "cuda")
        self.bp_check_every = max(1, int(bp_check_every))
        E = ctx.edges_number
        self.E = E
        self.half = E // 2
        # Storage bond dim: a bond dim in 5..15 that is not a multiple of 4 is stored zero-padded
        # to the next multiple of 4, so the register-tiled complex64 message kernels (built for
        # degrees 2-4 and chi in {4, 8, 12, 16}) serve every step.  Padding is exact: padded rows and
        # columns of tensors and messages stay zero, their singular values are 0 (masked and
        # sorted last, never counted by the truncation rank), and the truncation zeroes the
        # spectrum columns it drops.
        if pad_bonds is None:
            pad_bonds = self.precision == "single" and all(d <= 4 for d in ctx.degree_to_layout)
        self.pad_bonds = bool(pad_bonds)
        # BP sweeps in two stages (half-node message kernels + combine) on the complex64 path
        self.split_sweeps = self.precision == "single"
        chimax = self._store(ctx.max_bond_dim)
        if chimax > 32:
            raise NotImplementedError(
                f"max_bond_dim={chimax}: the truncation's Jacobi SVDs take 2*chi <= 64 (chi <= 32)")
        dev = self.device
        # classes whose node tensors exceed shared memory run on up to 8 CTAs per SM with work
        # tensors in this scratch (one buffer, shared: classes run one after another on the stream)
        n_ctas = 8 * torch.cuda.get_device_properties(self.device).multi_processor_count
        scratch_elems = 0
        for d, L in ctx.degree_to_layout.items():
            per_cta = int(self.lib.dll.bqa_node_scratch_elems(d, chimax, self.dtype))
            if per_cta:
                scratch_elems = max(scratch_elems, min(L.batch_size, n_ctas) * per_cta)
        self.scratch = torch.empty(scratch_elems, dtype=cplx, device=dev) if scratch_elems else None
        self.scratch_elems = scratch_elems
        i32 = torch.int32
        self.classes: list[_DeviceClass] = []
        for d, L in ctx.degree_to_layout.items():
            B = L.batch_size
            size = B * 2 * chimax ** d
            self.classes.append(_DeviceClass(
                degree=d, count=B,
                node_ids=torch.as_tensor(L.node_ids, dtype=i32, device=dev),
                in_pos=torch.as_tensor(np.ascontiguousarray(L.input_msgs_position.T), dtype=i32, device=dev),
                out_pos=torch.as_tensor(np.ascontiguousarray(L.output_msgs_position.T), dtype=i32, device=dev),
                lmbd_pos=torch.as_tensor(np.ascontiguousarray(L.lmbds_position.T), dtype=i32, device=dev),
                edge_ampl=torch.as_tensor(np.ascontiguousarray(np.asarray(L.edge_ampls, dtype=np.float64).T),
                                          dtype=torch.float64, device=dev),
                node_ampl=torch.as_tensor(L.node_ampls, dtype=torch.float64, device=dev),
                tensors=[torch.empty(size, dtype=cplx, device=dev) for _ in range(2)],
            ))
        nmax = 2 * chimax
        self.msgs = [torch.empty(E * chimax * chimax, dtype=cplx, device=dev) for _ in range(2)]
        # simple-update scratch: ext messages (later reused for canonicalisers), lu, ul
        self.ext = torch.empty(E * nmax * nmax, dtype=cplx, device=dev)
        self.lu = torch.empty(E * nmax * nmax, dtype=cplx, device=dev)
        self.ul = torch.empty(E * nmax * nmax, dtype=cplx, device=dev)
        self.lmbds = torch.empty(self.half * nmax, dtype=real, device=dev)
        # max over edges of each lambda column, as the real's bit pattern
        self.colmax = torch.zeros(nmax, dtype=torch.int32 if self.precision == "single" else torch.int64, device=dev)
        self.edge_j = torch.as_tensor(np.asarray(ctx.edge_ampl, dtype=np.float64), device=dev)
        self.dist_parts = torch.zeros(2, dtype=torch.int64, device=dev)
        self.loop_state = torch.zeros(8, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.rho = torch.empty(ctx.nodes_number * 4, dtype=cplx, device=dev)
        self.zz = torch.empty(self.half, dtype=torch.float64, device=dev)
        self.norm2 = torch.zeros(1, dtype=torch.float64, device=dev)
        self._plan_table = (ctypes.c_int32 * (33 * (len(self.classes) + 1)))()
        # Mixed-precision BP (mixed=True or BQA_GB300_MIXED=1, complex64): at storage bond dim 16
        # the degree-3 classes sweep with the mixed kernel (BQA_VARIANT_MIXED) -- BF16 tensor-core
        # sweeps while the BP distance is above the library's switch, FP32 sweeps after that, so
        # the run stops on an FP32 sweep at the reference tolerance
        if mixed is None:
            import os
            mixed = os.environ.get("BQA_GB300_MIXED", "0") == "1"
        self.mixed = bool(mixed) and self.precision == "single" and self.split_sweeps and any(
            c.degree == 3 for c in self.classes)
        if self.mixed:
            from .autotune import Plan
            chis = 16
            row = chis * (len(self.classes) + 1)
            variants = [_lib.BQA_VARIANT_MIXED if c.degree == 3 else _lib.BQA_VARIANT_DEFAULT for c in self.classes]
            self._plan_table[row] = 1
            for i, v in enumerate(variants):
                self._plan_table[row + 1 + i] = v
            self.plans[chis] = Plan(chis=chis, split=True, variants=variants)
        self.rng = np.random.default_rng(ctx.seed)
        self.stats: list[dict] = []
        self._events: list | None = None
        self.reset()

    def __del__(self):
        cache, self._graph_cache = getattr(self, "_graph_cache", None), None
        if cache is not None:
            try:
                self.lib.dll.bqa_graph_cache_destroy(cache)
            except Exception:
                pass

    def _graphs(self):
        """The job's BP graph cache (created on first use, with the job's device current)."""
        if self._graph_cache is None:
            h = ctypes.c_void_p()
            with self.torch.cuda.device(self.device):
                self.lib.call("bqa_graph_cache_create", ctypes.byref(h))
            self._graph_cache = h
        return self._graph_cache

    # ---- kernel timing (CUDA events on the launch stream) ----------------------------------
    def enable_kernel_timing(self, on: bool = True) -> None:
        """Record a CUDA event pair around every C-ABI launch group (bench instrumentation)."""
        self._events = [] if on else None

    def _launch(self, name: str, flops: float, nbytes: float, fn, *args) -> None:
        if self._events is None:
            fn(*args)
            return
        ev0 = self.torch.cuda.Event(enable_timing=True)
        ev1 = self.torch.cuda.Event(enable_timing=True)
        ev0.record()
        fn(*args)
        ev1.record()
        self._events.append([name, ev0, ev1, flops, nbytes])

    def kernel_times(self) -> list[tuple[str, float, float, float]]:
        """(name, milliseconds, algorithmic flops, algorithmic bytes) of every timed launch
        group since timing was enabled; synchronises the device."""
        if not self._events:
            return []
        self.torch.cuda.synchronize(self.device)
        return [(n, a.elapsed_time(b), f, by) for n, a, b, f, by in self._events]

    def bp_sweep_cost(self, chi: int | None = None) -> tuple[float, float]:
        """Algorithmic (flops, bytes) of one BP sweep at bond dim ``chi`` (the current one by
        default): per node of degree d, 2 d^2 chi^(d+1) complex MACs (d messages, each d-1 mode
        products and one closing contraction), and the tensor read once plus d messages read and d
        written."""
        chi = self.chi if chi is None else chi
        el = 8 if self.precision == "single" else 16
        f = b = 0.0
        for c in self.classes:
            if c.degree == 0:
                continue
            f += c.count * 8.0 * 2 * c.degree ** 2 * chi ** (c.degree + 1)
            b += c.count * el * (2.0 * chi ** c.degree + 2.0 * c.degree * chi * chi)
        return f, b

    # ---- helpers -------------------------------------------------------------------------
    def _store(self, chi: int) -> int:
        """Storage bond dim of logical bond dim ``chi``."""
        if self.pad_bonds and 4 < chi <= 16 and chi % 4:
            return chi + 4 - chi % 4
        return chi

    @property
    def stream(self) -> int:
        return self.torch.cuda.current_stream(self.device).cuda_stream

    def _class_array(self, out: bool = False):
        arr = (_lib.BqaClass * len(self.classes))()
        for i, c in enumerate(self.classes):
            arr[i] = _lib.BqaClass(
                c.degree, c.count, _ptr(c.node_ids), _ptr(c.in_pos), _ptr(c.out_pos), _ptr(c.lmbd_pos),
                _ptr(c.edge_ampl), _ptr(c.node_ampl), _ptr(c.tensors[self.tcur]),
                _ptr(c.tensors[1 - self.tcur]) if out else 0,
                _ptr(self.scratch) if self.scratch is not None else 0, self.scratch_elems)
        return arr

    @property
    def _np_cplx(self):
        return np.complex64 if self.precision == "single" else np.complex128

    @property
    def bond_dim(self) -> int:
        return self.chi

    def _msgs_cur(self):
        return self.msgs[self.mcur]

    # ---- state -----------------------------------------------------------------------------
    def reset(self) -> None:
        """Initial product state (src/bqa/state.py:41-74): every tensor [sqrt(.5), -sqrt(.5)],
        bond dim 1, lambdas 1, messages diag(lambda)/tr."""
        self.chi = self.chis = 1
        self.tcur = 0
        self.mcur = 0
        self.blocks_valid = False
        init = self.torch.tensor([complex(INIT_STATE[0]), complex(INIT_STATE[1])], dtype=self.msgs[0].dtype,
                                 device=self.device)
        for c in self.classes:
            c.tensors[0][: 2 * c.count].view(c.count, 2).copy_(init.expand(c.count, 2))
        self.lam_stride = 1
        self.lmbds[: self.half].fill_(1.0)
        self.lib.call("bqa_msgs_from_lmbds", _ptr(self.lmbds), 1, self.E, 1, self.dtype, _ptr(self._msgs_cur()),
                      self.stream)

    def set_state(self, degree_to_tensor: dict, msgs: np.ndarray, lmbds: np.ndarray | None = None) -> None:
        """Load a state given as numpy arrays (tensors ``(B, 2, chi, ..)`` per degree, messages
        ``(E, chi, chi)``, optional lambdas ``(E/2, chi)``); the bond dim is taken from msgs."""
        torch = self.torch
        chi = int(msgs.shape[-1])
        if chi > self.ctx.max_bond_dim:
            raise ValueError("state bond dim exceeds max_bond_dim")
        chis = self._store(chi)
        self.chi, self.chis, self.tcur, self.mcur = chi, chis, 0, 0
        self.blocks_valid = False
        for c in self.classes:
            t = np.asarray(degree_to_tensor[c.degree], dtype=self._np_cplx)
            if chis != chi:
                t = np.pad(t, [(0, 0), (0, 0)] + [(0, chis - chi)] * c.degree)
            t = np.ascontiguousarray(t).reshape(-1)
            c.tensors[0][: t.size].copy_(torch.from_numpy(t))
        m = np.asarray(msgs, dtype=self._np_cplx)
        if chis != chi:
            m = np.pad(m, [(0, 0), (0, chis - chi), (0, chis - chi)])
        m = np.ascontiguousarray(m).reshape(-1)
        self.msgs[0][: m.size].copy_(torch.from_numpy(m))
        if lmbds is not None:
            lam = np.ascontiguousarray(lmbds.real, dtype=self.real_np)
            self.lam_stride = lam.shape[1]
            self.lmbds[: lam.size].copy_(torch.from_numpy(lam.reshape(-1)))

    def snapshot(self) -> dict:
        """Device-side copy of the evolving state (current tensors, messages, lambdas, bond
        dims, host RNG); ``restore`` puts it back, so a run can resume from this point."""
        n_t = {id(c): c.count * 2 * self.chis ** c.degree for c in self.classes}
        return {
            "tensors": [c.tensors[self.tcur][: n_t[id(c)]].clone() for c in self.classes],
            "msgs": self._msgs_cur()[: self.E * self.chis * self.chis].clone(),
            "lmbds": self.lmbds.clone(),
            "dims": (self.chi, self.chis, self.lam_stride),
            "rng": self.rng.bit_generator.state,
        }

    def restore(self, snap: dict) -> None:
        self.chi, self.chis, self.lam_stride = snap["dims"]
        self.tcur, self.mcur = 0, 0
        self.blocks_valid = False
        for c, t in zip(self.classes, snap["tensors"]):
            c.tensors[0][: t.numel()].copy_(t)
        self.msgs[0][: snap["msgs"].numel()].copy_(snap["msgs"])
        self.lmbds.copy_(snap["lmbds"])
        self.rng.bit_generator.state = snap["rng"]

    def get_state(self) -> tuple[dict, np.ndarray, np.ndarray]:
        """Numpy copies of (tensors per degree, messages (E, chi, chi), lambdas (E/2, chi))."""
        chi, chis = self.chi, self.chis
        tens = {}
        for c in self.classes:
            shape = (c.count, 2) + (chis,) * c.degree
            t = c.tensors[self.tcur][: int(np.prod(shape))].cpu().numpy().reshape(shape)
            tens[c.degree] = t[(slice(None), slice(None)) + (slice(0, chi),) * c.degree]
        msgs = self._msgs_cur()[: self.E * chis * chis].cpu().numpy().reshape(self.E, chis, chis)[:, :chi, :chi]
        lam = self.lmbds[: self.half * self.lam_stride].cpu().numpy().reshape(self.half, self.lam_stride)[:, :chi]
        return tens, msgs, lam

    # ---- annealing step --------------------------------------------------------------------
    def gate_layer(self, xtime: float, ztime: float) -> tuple[int, float]:
        """ZZ layer with BP-gauged truncation (``_simple_update``, src/bqa/state.py:230-247),
        then the Rz and Rx layers and the symmetric gauge (state.py:142-156,219-227), fused:
        extended messages -> environment factors -> bond canonicalisers and lambdas ->
        global truncation dim (one small device-to-host read) -> tensor update ->
        messages diag(lambda)/tr.  Returns (new bond dim, truncation error bound)."""
        lib, st = self.lib, self.stream
        ctx = self.ctx
        chi = self.chis
        n = 2 * chi
        eps = float(ctx.pinv_eps)
        cls = self._class_array()
        dt = self.dtype
        if self.split_sweeps and self.blocks_valid and self.reuse_blocks:
            # the converged BP run left the open-bond blocks of these messages in lu
            self._launch("ext_msgs", 0.0, 0.0, lib.call, "bqa_ext_combine", _ptr(self.lu), self.E, chi, dt,
                         _ptr(self.edge_j), float(ztime), _ptr(self.ext), st)
        elif self.split_sweeps:
            # half-node kernels write P_0, P_1 into lu (free until the environment factors)
            self._launch("ext_msgs", 0.0, 0.0, lib.call, "bqa_ext_msgs_split", cls, len(self.classes), chi, dt,
                         _ptr(self._msgs_cur()), _ptr(self.lu), self.E, _ptr(self.edge_j), float(ztime),
                         _ptr(self.ext), st)
        else:
            self._launch("ext_msgs", 0.0, 0.0, lib.call, "bqa_ext_msgs", cls, len(self.classes), chi, dt,
                         _ptr(self._msgs_cur()), _ptr(self.ext), float(ztime), st)
        self.blocks_valid = False
        self._launch("env_factor", 0.0, 0.0, lib.call, "bqa_env_factor", _ptr(self.ext), self.E, n, dt, eps,
                     _ptr(self.lu), _ptr(self.ul), _ptr(self.status), st)
        self.colmax.zero_()
        canon = self.ext  # the extended messages are consumed; reuse their storage
        self._launch("bond_canon", 0.0, 0.0, lib.call, "bqa_bond_canon", _ptr(self.lu), _ptr(self.ul), self.E, n,
                     dt, eps, _ptr(canon), _ptr(self.lmbds), _ptr(self.colmax), _ptr(self.status), st)
        # global truncation (src/bqa/backends.py:297-303)
        max_l = self.colmax[:n].view(self.lmbds.dtype).cpu().numpy().astype(np.float64)
        if int(self.status.item()):
            log.warning("a Jacobi SVD of the truncation step hit its sweep cap")
            self.status.zero_()
        rank = n - int(np.sum(max_l < eps))
        dim = min(rank, ctx.max_bond_dim)
        err = float(np.sqrt(np.sum(max_l[dim:] ** 2)))
        log.info(f"Truncation performed, per edge error upper bound: {err}")
        dims = self._store(dim)
        if dims != dim:
            # padded storage: the spectrum columns the truncation drops become exact zeros
            lib.call("bqa_lmbds_truncate", _ptr(self.lmbds), n, self.half, dim, dt, st)
        cls = self._class_array(out=True)
        self._launch("apply_update", 0.0, 0.0, lib.call, "bqa_apply_update", cls, len(self.classes), chi, dims, dt,
                     _ptr(canon), _ptr(self.lmbds), n, float(ztime), float(xtime), st)
        self.tcur = 1 - self.tcur
        self.chi, self.chis = dim, dims
        self.lam_stride = n
        lib.call("bqa_msgs_from_lmbds", _ptr(self.lmbds), n, self.E, dims, dt, _ptr(self._msgs_cur()), st)
        return dim, err

    def run_layer(self, xtime: float, ztime: float) -> dict:
        """One annealing step (src/bqa/state.py:315-321)."""
        if self.native and self._events is None:
            info = self._run_layer_native(float(xtime), float(ztime))
        else:
            dim, err = self.gate_layer(xtime, ztime)
            sweeps = self.run_bp()
            info = {"bond_dim": dim, "trunc_err": err, "sweeps": sweeps}
            self.stats.append(info)
        if self.autotune and self.chis not in self.plans:
            self.tune()
        return info

    def tune(self):
        """Time the BP message-kernel candidates at the current bond dim on the live state and
        use the fastest from the next sweep on (autotune.tune); returns the plan."""
        from . import autotune
        self.blocks_valid = False   # the candidate sweeps write lu
        plan = autotune.tune(self)
        self.plans[self.chis] = plan
        row = self.chis * (len(self.classes) + 1)
        self._plan_table[row] = 1 if plan.split else 2
        for i, v in enumerate(plan.variants):
            self._plan_table[row + 1 + i] = int(v)
        return plan

    def _plan_row(self):
        """(two-stage?, variants array) of the current bond dim's plan, or None."""
        if self.chis not in self.plans:
            return None
        row = self.chis * (len(self.classes) + 1)
        arr = (ctypes.c_int32 * len(self.classes)).from_buffer(self._plan_table, 4 * (row + 1))
        return self._plan_table[row] == 1, arr

    def _job_struct(self):
        ctx = self.ctx
        cls = self._class_array(out=True)          # tensor = current buffer, tensor_out = the other
        j = _lib.BqaJob()
        j.dtype, j.n_classes = self.dtype, len(self.classes)
        j.classes = ctypes.cast(cls, ctypes.POINTER(_lib.BqaClass))
        j.edges, j.max_bond_dim = self.E, int(ctx.max_bond_dim)
        j.max_bp_iters, j.bp_check_every = int(ctx.max_bp_iters_number), self.bp_check_every
        j.pad_bonds, j.split_sweeps = int(self.pad_bonds), int(self.split_sweeps)
        j.colmax_elems = int(self.colmax.numel())
        j.chi, j.chis, j.lam_stride, j.mcur, j.tcur = self.chi, self.chis, self.lam_stride, self.mcur, self.tcur
        j.bp_eps, j.pinv_eps, j.damping = float(ctx.bp_eps), float(ctx.pinv_eps), float(ctx.damping)
        j.msgs[0], j.msgs[1] = _ptr(self.msgs[0]), _ptr(self.msgs[1])
        j.ext, j.lu, j.ul, j.lmbds = _ptr(self.ext), _ptr(self.lu), _ptr(self.ul), _ptr(self.lmbds)
        j.colmax, j.dist_parts = _ptr(self.colmax), _ptr(self.dist_parts)
        j.loop_state, j.status, j.edge_j = _ptr(self.loop_state), _ptr(self.status), _ptr(self.edge_j)
        if self.plans:
            j.sweep_variants = ctypes.cast(self._plan_table, ctypes.POINTER(ctypes.c_int32))
        j.blocks_valid = int(self.blocks_valid and self.reuse_blocks)
        return j, cls

    def _run_layer_native(self, xtime: float, ztime: float) -> dict:
        if self.ctx.max_bp_iters_number < 1:
            raise ValueError("max_bp_iter_number must be >= 1 to run belief propagation")
        j, cls = self._job_struct()
        res = _lib.BqaLayerInfo()
        if self.graphs:
            self.lib.call("bqa_run_layer_graph", ctypes.byref(j), self._graphs(), xtime, ztime, ctypes.byref(res),
                          self.stream)
        else:
            self.lib.call("bqa_run_layer", ctypes.byref(j), xtime, ztime, ctypes.byref(res), self.stream)
        return self._adopt(j, res)

    def run_layer_packed(self, xtime: float, ztime: float, packer) -> dict:
        """One step whose BP run is swept together with other jobs' (``packer``: a
        ``serve.BpPacker``, or a function from the sweep's FLOPs at the new bond dim to one): the
        gate layer through bqa_gate_layer on this job's stream, then the BP run in the packer's
        shared launches.  The state afterwards is the same bits as after ``run_layer``."""
        if self.ctx.max_bp_iters_number < 1:
            raise ValueError("max_bp_iter_number must be >= 1 to run belief propagation")
        j, cls = self._job_struct()
        res = _lib.BqaLayerInfo()
        self.lib.call("bqa_gate_layer", ctypes.byref(j), xtime, ztime, ctypes.byref(res), self.stream)
        self.torch.cuda.current_stream(self.device).synchronize()
        if not hasattr(packer, "run_bp"):
            packer = packer(self.bp_sweep_cost(int(j.chi))[0])
        packer.run_bp(j, res)
        return self._adopt(j, res)

    def _adopt(self, j, res) -> dict:
        """Take over the job struct's state after a native step and log / record its figures."""
        self.chi, self.chis, self.lam_stride, self.mcur, self.tcur = j.chi, j.chis, j.lam_stride, j.mcur, j.tcur
        self.blocks_valid = bool(j.blocks_valid)
        if res.svd_not_converged:
            log.warning("a Jacobi SVD of the truncation step hit its sweep cap")
        log.info(f"Truncation performed, per edge error upper bound: {res.trunc_err}")
        if res.bp_exhausted:
            log.warning(f"BP algorithm exceeds iterations limit set to {self.ctx.max_bp_iters_number}, "
                        f"obtained bp_eps {res.best_dist}")
        info = {"bond_dim": int(res.bond_dim), "trunc_err": float(res.trunc_err), "sweeps": int(res.sweeps)}
        self.stats.append(info)
        return info

    def run_bp(self) -> int:
        """Loopy BP to tolerance (src/bqa/state.py:97-124).  Sweeps are launched in groups of
        ``bp_check_every`` between host checks; sweeps queued after convergence return at once
        on the device.  Returns the number of sweeps run."""
        ctx = self.ctx
        if ctx.max_bp_iters_number < 1:
            raise ValueError("max_bp_iter_number must be >= 1 to run belief propagation")
        if self.native and self.graphs and self._events is None:
            return self._run_bp_graph()
        lib, st = self.lib, self.stream
        cls = self._class_array()
        a, b = self.msgs[self.mcur], self.msgs[1 - self.mcur]
        self.loop_state.zero_()
        self.dist_parts.zero_()
        elems = self.E * self.chis * self.chis
        launched = 0
        eps, damp = float(ctx.bp_eps), float(ctx.damping)
        flops, nbytes = self.bp_sweep_cost()
        first = len(self._events) if self._events is not None else 0
        plan = self._plan_row()
        while True:
            for _ in range(min(self.bp_check_every, ctx.max_bp_iters_number - launched)):
                if plan is not None:
                    self._launch("bp_sweep", flops, nbytes, lib.call, "bqa_bp_sweep_plan", cls, len(self.classes),
                                 self.chis, self.dtype, plan[1], _ptr(a), _ptr(b), _ptr(self.lu) if plan[0] else None,
                                 self.E, _ptr(self.dist_parts), _ptr(self.loop_state), st)
                elif self.split_sweeps:
                    # open-bond blocks into the idle simple-update scratch, then the messages
                    self._launch("bp_sweep", flops, nbytes, lib.call, "bqa_bp_sweep_split", cls, len(self.classes),
                                 self.chis, self.dtype, _ptr(a), _ptr(b), _ptr(self.lu), self.E,
                                 _ptr(self.dist_parts), _ptr(self.loop_state), st)
                else:
                    self._launch("bp_sweep", flops, nbytes, lib.call, "bqa_bp_sweep", cls, len(self.classes),
                                 self.chis, self.dtype, _ptr(a), _ptr(b), _ptr(self.dist_parts),
                                 _ptr(self.loop_state), st)
                lib.call("bqa_bp_finalize", _ptr(a), _ptr(b), elems, self.dtype, _ptr(self.dist_parts),
                         _ptr(self.loop_state), eps, damp, ctx.max_bp_iters_number, st)
                launched += 1
            ls = self.loop_state.cpu().numpy()
            if ls[0]:
                break
            if launched >= ctx.max_bp_iters_number:
                raise RuntimeError("BP loop state did not finish after the iteration cap")
        if self._events is not None:
            # sweeps queued after convergence returned at once: they did no algorithmic work
            sw = [e for e in self._events[first:] if e[0] == "bp_sweep"]
            for e in sw[int(ls[1]):]:
                e[0] = "bp_sweep_skipped"
        if ls[2]:
            self.mcur = 1 - self.mcur
        two_stage = plan[0] if plan is not None else self.split_sweeps
        self.blocks_valid = not ls[3] and bool(two_stage)
        if ls[3]:
            best = np.array([ls[6]], dtype=np.int32).view(np.float32)[0]
            log.warning(f"BP algorithm exceeds iterations limit set to {ctx.max_bp_iters_number}, "
                        f"obtained bp_eps {best}")
        return int(ls[1])

    def _run_bp_graph(self) -> int:
        j, cls = self._job_struct()
        res = _lib.BqaLayerInfo()
        self.lib.call("bqa_run_bp_graph", ctypes.byref(j), self._graphs(), ctypes.byref(res), self.stream)
        self.mcur = j.mcur
        self.blocks_valid = bool(j.blocks_valid)
        if res.bp_exhausted:
            log.warning(f"BP algorithm exceeds iterations limit set to {self.ctx.max_bp_iters_number}, "
                        f"obtained bp_eps {res.best_dist}")
        return int(res.sweeps)

    # ---- read-out ------------------------------------------------------------------------
    def density_matrices(self) -> np.ndarray:
        """(n, 2, 2) complex marginals (src/bqa/state.py:77-94)."""
        self.lib.call("bqa_densities", self._class_array(), len(self.classes), self.chis, self.dtype,
                      _ptr(self._msgs_cur()), _ptr(self.rho), self.stream)
        return self.rho.view(-1, 2, 2).cpu().numpy().astype(np.complex128)

    def bloch_vectors(self) -> np.ndarray:
        rho = self.density_matrices()
        x = (rho[:, 0, 1] + rho[:, 1, 0]).real
        y = (rho[:, 1, 0] - rho[:, 0, 1]).imag
        z = (rho[:, 0, 0] - rho[:, 1, 1]).real
        return np.stack([x, y, z], axis=1)

    def edge_zz(self) -> np.ndarray:
        """BP two-site <Z_u Z_v> per undirected edge (oracle ``edge_zz``)."""
        pm = self.lu   # scratch of the simple update, idle between steps
        self.blocks_valid = False
        self.lib.call("bqa_psplit", self._class_array(), len(self.classes), self.chis, self.dtype,
                      _ptr(self._msgs_cur()), _ptr(pm), self.stream)
        self.lib.call("bqa_edge_zz", _ptr(pm), self.E, self.chis, self.dtype, _ptr(self.zz), self.stream)
        return self.zz.cpu().numpy()

    def energy(self, zz: np.ndarray | None = None, z: np.ndarray | None = None) -> float:
        ctx = self.ctx
        zz = self.edge_zz() if zz is None else zz
        z = self.bloch_vectors()[:, 2] if z is None else z
        return float(np.dot(ctx.edge_ampl, zz) + np.dot(ctx.node_ampl, z))

    def spin_readout(self, z: np.ndarray | None = None) -> np.ndarray:
        """Deterministic read-out sign(<Z_i>) -> +1 / -1 (z > 0 -> +1)."""
        z = self.bloch_vectors()[:, 2] if z is None else z
        return np.where(z > 0, 1, -1)

    def spin_energy(self, spins: np.ndarray) -> float:
        ctx = self.ctx
        return float(np.dot(ctx.edge_ampl, spins[ctx.edge_src] * spins[ctx.edge_dst]) + np.dot(ctx.node_ampl, spins))

    # ---- measurement -----------------------------------------------------------------------
    def _project(self, nodes, outcomes) -> None:
        """Project nodes onto outcomes (0: |0>, 1: |1>), then renormalise each touched class."""
        ctx = self.ctx
        self.blocks_valid = False
        nodes = np.asarray(nodes, dtype=np.int64)
        outcomes = np.asarray(outcomes, dtype=np.int64)
        deg = ctx.node_degree[nodes]
        for i, c in enumerate(self.classes):
            sel = deg == c.degree
            if not np.any(sel):
                continue
            pos = self.torch.as_tensor(ctx.node_position[nodes[sel]].astype(np.int32), device=self.device)
            out = self.torch.as_tensor(outcomes[sel].astype(np.int32), device=self.device)
            self.lib.call("bqa_project_nodes", _ptr(c.tensors[self.tcur]), c.count, 2 * self.chis ** c.degree,
                          self.dtype, _ptr(pos), _ptr(out), int(pos.numel()), _ptr(self.norm2), self.stream)

    def measure(self) -> list:
        """Sequential most-polarised-first sampling (src/bqa/state.py:250-312) with the same
        host generator (numpy default_rng(seed).uniform) and the same order of draws."""
        ctx = self.ctx
        n = ctx.nodes_number
        thr = ctx.measurement_threshold
        result = np.zeros(n, dtype=np.int64)
        measured = np.zeros(n, dtype=bool)
        while not measured.all():
            probs = self.density_matrices()[:, 0, 0].real
            free = np.flatnonzero(~measured)
            node = int(free[np.argmax(np.abs(2.0 * probs[free] - 1.0))])
            prob = float(probs[node])
            outcome = 0 if prob > self.rng.uniform(0.0, 1.0) else 1
            self._project([node], [outcome])
            measured[node] = True
            result[node] = 1 - 2 * outcome
            self.run_bp()
            probs = self.density_matrices()[:, 0, 0].real
            free = np.flatnonzero(~measured)
            up = free[probs[free] > thr]
            down = free[probs[free] < 1.0 - thr]
            batch = np.concatenate([up, down])
            if batch.size:
                self._project(batch, np.concatenate([np.zeros(up.size, np.int64), np.ones(down.size, np.int64)]))
                measured[batch] = True
                result[up] = 1
                result[down] = -1
            self.run_bp()
        log.info("Measurement outcomes sampling completed")
        return [int(x) for x in result]
