"""CPU oracle for the bqa annealing hot path -- TEST INFRASTRUCTURE ONLY.

This module is the oracle, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.  The GB300 package never calls it
and has no CPU fallback.

It is a numpy restatement of the reference numpy backend's algorithm (LuchnikovI/bqa
v0.1.6), in the same batched order of operations and at the same precision
(complex128 by default = the reference at ``BQA_PRECISION=double``; complex64 =
``single``).  Each function cites the reference lines it follows.  It is pinned against
the reference itself: ``tests/golden/make_golden.py`` imports the reference and records
its outputs, and ``tests/test_oracle_golden.py`` checks this module against them.

Additions the reference does not have, defined here once and used as the definition for
the device kernels: the BP two-site estimate of <Z_i Z_j> on an edge, and the energy
``sum_ij J_ij <Z_i Z_j> + sum_i h_i <Z_i>`` (sign convention of the gates in
``src/bqa/exact_sim.py:36-43``).
"""
from __future__ import annotations

import logging
from dataclasses import dataclass
from math import cos, inf, sin, sqrt

import numpy as np

from bqa_gb300 import config as cfg

log = logging.getLogger(__name__)

# src/bqa/backends.py:20-22
SQRT_NEG_1J = sqrt(2.0) / 2.0 - 1j * sqrt(2.0) / 2.0
SQRT_1J = sqrt(2.0) / 2.0 + 1j * sqrt(2.0) / 2.0


# ----------------------------------------------------------------------------------------
# degree-class layout, restated as the reference's per-node loop
# (src/bqa/config/config_canonicalization.py:62-131, 171-249)
# ----------------------------------------------------------------------------------------

@dataclass
class OracleLayout:
    node_ids: np.ndarray
    input_msgs_position: list
    output_msgs_position: list
    lmbds_position: list
    node_ampls: np.ndarray
    edge_ampls: list


@dataclass
class OracleContext:
    graph: list
    nodes_number: int
    edges_number: int
    max_bond_dim: int
    max_bp_iters_number: int
    bp_eps: float
    pinv_eps: float
    measurement_threshold: float
    damping: float
    seed: int
    instructions: list
    degree_to_layout: dict
    path_to_tensors: dict
    edge_to_ampl: dict
    node_to_ampl: dict
    edge_to_msg_pos: dict
    edge_to_lmbd_pos: dict
    dtype: type

    @property
    def lmbds_number(self):
        return self.edges_number // 2

    @property
    def msg_pos_to_lmbd_pos(self):
        return np.arange(self.edges_number) % self.lmbds_number


def make_context(config: dict, dtype=np.complex128) -> OracleContext:
    c = cfg.analyse_config(config)
    edges = c[cfg.EDGES_KEY]
    n = 1 + max(max(c[cfg.NODES_KEY].keys(), default=-1),
                max(max(a, b) for a, b in edges.keys()))
    graph = [[] for _ in range(n)]
    for a, b in edges.keys():                                      # :182-186
        graph[a].append(b)
    msg_pos = {e: p for p, e in enumerate(edges.keys())}            # :189-190
    half = len(edges) // 2
    lmbd_pos = {e: p % half for p, e in enumerate(edges.keys())}    # :194-196
    node_to_ampl = {v: c[cfg.NODES_KEY].get(v, c[cfg.DEFAULT_FIELD_KEY]) for v in range(n)}
    raw: dict = {}
    for v, nbrs in enumerate(graph):                                # :87-107
        d = len(nbrs)
        if d not in raw:
            raw[d] = dict(ids=[], inp=[[] for _ in range(d)], out=[[] for _ in range(d)],
                          lam=[[] for _ in range(d)], na=[], ea=[[] for _ in range(d)])
        L = raw[d]
        L["ids"].append(v)
        L["na"].append(node_to_ampl[v])
        for k, u in enumerate(nbrs):
            L["inp"][k].append(msg_pos[(u, v)])
            L["out"][k].append(msg_pos[(v, u)])
            L["lam"][k].append(lmbd_pos[(v, u)])
            L["ea"][k].append(edges[(v, u)])
    layouts = {
        d: OracleLayout(
            np.array(L["ids"], dtype=np.intp),
            [np.array(x, dtype=np.intp) for x in L["inp"]],
            [np.array(x, dtype=np.intp) for x in L["out"]],
            [np.array(x, dtype=np.intp) for x in L["lam"]],
            np.array(L["na"], dtype=np.float64),
            [np.array(x, dtype=np.float64) for x in L["ea"]],
        ) for d, L in raw.items()
    }
    paths = {int(v): (d, pos) for d, L in layouts.items() for pos, v in enumerate(L.node_ids)}
    return OracleContext(
        graph, n, len(edges), c[cfg.MAX_BOND_DIM_KEY], c[cfg.MAX_BP_ITER_NUMBER_KEY],
        c[cfg.BP_EPS_KEY], c[cfg.PINV_EPS_KEY], c[cfg.MEASUREMENT_THRESHOLD_KEY],
        c[cfg.DAMPING_KEY], c[cfg.SEED_KEY], cfg.canonicalize_schedule(c[cfg.SCHEDULE_KEY]),
        layouts, paths, edges, node_to_ampl, msg_pos, lmbd_pos, dtype)


# ----------------------------------------------------------------------------------------
# batched tensor helpers: tensors are (B, 2, b_0, ..., b_{d-1}); messages (B, chi, chi)
# ----------------------------------------------------------------------------------------

def _bcast(v: np.ndarray, rank: int) -> np.ndarray:
    return v.reshape((-1,) + (1,) * (rank - 1))


def _apply_first_bond(t: np.ndarray, m: np.ndarray) -> np.ndarray:
    """``tensordot(t, m, [[1],[1]])`` per batch item: contract the first bond with the
    message's column index, append the new index last (src/bqa/backends.py:381-391)."""
    B, chi_in = t.shape[0], t.shape[2]
    moved = np.moveaxis(t, 2, -1)
    out = moved.reshape(B, -1, chi_in) @ np.swapaxes(m, 1, 2)
    return out.reshape(moved.shape[:-1] + (m.shape[1],))


def _rotate_first_bond(t: np.ndarray) -> np.ndarray:
    return np.moveaxis(t, 2, -1)                                   # backends.py:376-379


def _z_phys(t: np.ndarray) -> np.ndarray:
    out = t.copy()                                                 # backends.py:635-639
    out[:, 1] *= -1.0
    return out


def _x_phys(t: np.ndarray) -> np.ndarray:
    return t[:, ::-1]                                              # backends.py:631-633


def _extend_bond(t: np.ndarray, raw_axis: int, coupling: np.ndarray, conj: bool) -> np.ndarray:
    """Half of exp(-i c Z Z) on one bond, doubling it (src/bqa/backends.py:519-526).

    ``coupling`` is complex-typed like the reference's, so cos/sqrt follow numpy's
    complex branch conventions exactly.
    """
    c = coupling.astype(t.dtype)
    a0 = np.sqrt(np.cos(c))
    a1 = np.sqrt(np.sin(c))
    if conj:
        up = t * _bcast(np.conj(a0), t.ndim)
        down = _z_phys(t) * _bcast(SQRT_1J * np.conj(a1), t.ndim)
    else:
        up = t * _bcast(a0, t.ndim)
        down = _z_phys(t) * _bcast(SQRT_NEG_1J * a1, t.ndim)
    return np.concatenate([up, down], axis=raw_axis)


def _contract_all_but(lhs: np.ndarray, rhs: np.ndarray, raw_axis: int) -> np.ndarray:
    """out[a, b] = sum over every batch axis but ``raw_axis`` of lhs[.., a, ..] rhs[.., b, ..]."""
    B = lhs.shape[0]
    l2 = np.moveaxis(lhs, raw_axis, 1).reshape(B, lhs.shape[raw_axis], -1)
    r2 = np.moveaxis(rhs, raw_axis, 1).reshape(B, rhs.shape[raw_axis], -1)
    return l2 @ np.swapaxes(r2, 1, 2)


def _trace_normalize(m: np.ndarray) -> np.ndarray:
    return m / np.trace(m, axis1=-2, axis2=-1)[:, None, None]      # backends.py:316-318


def _apply_msgs_but_one(t: np.ndarray, msgs: list, idx: int) -> np.ndarray:
    for k, m in enumerate(msgs):                                   # backends.py:381-391
        t = _rotate_first_bond(t) if k == idx else _apply_first_bond(t, m)
    return t


def pass_msgs(t: np.ndarray, msgs: list, times: list | None = None) -> list:
    """Outgoing messages of a degree class (src/bqa/backends.py:393-408)."""
    tc = np.conj(t)
    out = []
    for idx in range(len(msgs)):
        tm = _apply_msgs_but_one(t, msgs, idx)
        tcc = tc
        if times is not None:
            tm = _extend_bond(tm, idx + 2, times[idx], conj=False)
            tcc = _extend_bond(tc, idx + 2, times[idx], conj=True)
        out.append(_trace_normalize(_contract_all_but(tcc, tm, idx + 2)))
    return out


def psplit_msgs(t: np.ndarray, msgs: list) -> list:
    """Per bond idx the phys-resolved open-bond blocks ``P_s[a,b]`` (s = 0, 1), unnormalised:
    ``P_s = sum conj(T)[s,..,a,..] (T x_{k!=idx} M_k)[s,..,b,..]``.  The BP message of
    ``pass_msgs`` is ``(P_0 + P_1)/tr``; used for the two-site <Z Z> estimate."""
    tc = np.conj(t)
    out = []
    for idx in range(len(msgs)):
        tm = _apply_msgs_but_one(t, msgs, idx)
        ps = [_contract_all_but(tc[:, s:s + 1], tm[:, s:s + 1], idx + 2) for s in (0, 1)]
        out.append(np.stack(ps, axis=1))      # (B, 2, chi, chi)
    return out


# ----------------------------------------------------------------------------------------
# state VM (src/bqa/state.py)
# ----------------------------------------------------------------------------------------

@dataclass
class OracleState:
    rng: np.random.Generator
    degree_to_tensor: dict
    msgs: np.ndarray
    lmbds: np.ndarray

    @property
    def bond_dim(self) -> int:
        # the lambdas carry the global bond dim for every degree class, also degree 0
        return int(self.lmbds.shape[1])


def _msgs_from_lmbds(lmbds: np.ndarray, ctx: OracleContext) -> np.ndarray:
    lam = lmbds[ctx.msg_pos_to_lmbd_pos]                           # state.py:56-57
    diag = lam[..., None] * np.eye(lam.shape[-1], dtype=lam.dtype)
    return _trace_normalize(diag)


def initialize_state(ctx: OracleContext) -> OracleState:
    dt = ctx.dtype                                                 # state.py:21-74
    init = np.array([np.sqrt(0.5), -np.sqrt(0.5)], dt)
    tensors = {d: np.broadcast_to(init.reshape((2,) + (1,) * d), (L.node_ids.shape[0], 2) + (1,) * d).copy()
               for d, L in ctx.degree_to_layout.items()}
    lmbds = np.ones((ctx.lmbds_number, 1), dt)
    return OracleState(np.random.default_rng(ctx.seed), tensors, _msgs_from_lmbds(lmbds, ctx), lmbds)


def get_dist(new: np.ndarray, old: np.ndarray) -> float:
    return float(np.abs(new - old).max() / np.abs(new + old).max())   # backends.py:492-495


def run_bp(ctx: OracleContext, st: OracleState) -> int:
    """Loopy BP to tolerance (src/bqa/state.py:97-124).  Returns the sweeps run.

    On convergence the messages of the PREVIOUS sweep are kept (:118-120); on exhaustion
    the raw output of the last sweep is kept, because ``best_msgs`` aliases the reused
    output buffer (:104,115,122-123)."""
    best = inf
    chi = st.bond_dim
    new = np.empty((ctx.edges_number, chi, chi), ctx.dtype)
    for it in range(ctx.max_bp_iters_number):
        for d, t in st.degree_to_tensor.items():
            L = ctx.degree_to_layout[d]
            aligned = [st.msgs[p] for p in L.input_msgs_position]
            for m, p in zip(pass_msgs(t, aligned), L.output_msgs_position):
                new[p] = m
        dist = get_dist(new, st.msgs)
        best = min(best, dist)
        if dist < ctx.bp_eps:
            return it + 1
        st.msgs *= ctx.damping                                     # backends.py:762-764
        st.msgs += (1.0 - ctx.damping) * new
    st.msgs = new
    log.warning(f"BP algorithm exceeds iterations limit set to {ctx.max_bp_iters_number}, obtained bp_eps {best}")
    return ctx.max_bp_iters_number


def _masked_svd(m: np.ndarray, eps: float):
    u, s, vh = np.linalg.svd(m, full_matrices=False)               # backends.py:709-717
    mask = s > eps
    return u * mask[:, None, :], s * mask, vh * mask[:, :, None]


def get_canonicalizers(msgs: np.ndarray, eps: float):
    """BP-gauged bond factorisation (src/bqa/state.py:171-200, backends.py:483-490).

    Returns lambdas ``(E/2, n)`` (real, descending, L2-normalised per edge) and the
    canonicalisers ``(E, n, n)``: slot ``p < E/2`` holds the one for the destination of
    forward edge p, slot ``p + E/2`` the one for its source."""
    E = msgs.shape[0]
    half = E // 2
    u, s, vh = _masked_svd(msgs, eps)
    sq = np.sqrt(s.astype(msgs.dtype))
    lu = sq[:, :, None] * vh
    inv = np.zeros_like(sq)
    nz = sq.real > np.finfo(msgs.dtype).eps                        # backends.py:719-727
    inv[nz] = 1.0 / sq[nz]
    ul = u * inv[:, None, :]
    ker = lu[:half] @ np.swapaxes(lu[half:], 1, 2)
    us, lam, vhs = _masked_svd(ker, eps)
    vs = np.swapaxes(vhs, 1, 2)
    can = np.concatenate([ul[half:] @ vs, ul[:half] @ us], axis=0)
    lam = lam / np.linalg.norm(lam, axis=1, keepdims=True)
    return lam, can


def truncation_dim(lmbds: np.ndarray, max_dim: int, eps: float) -> tuple[int, float]:
    """Global bond dim after truncation and the per-edge error bound (backends.py:297-303)."""
    max_l = np.abs(lmbds.real.max(axis=0))
    rank = max_l.shape[0] - int(np.sum(max_l < eps))
    dim = min(rank, max_dim)
    return dim, float(np.sqrt(np.sum(max_l[dim:] ** 2)))


def get_extended_msgs(ctx: OracleContext, ztime: float, st: OracleState) -> np.ndarray:
    chi = st.bond_dim                                              # state.py:127-139
    new = np.empty((ctx.edges_number, 2 * chi, 2 * chi), ctx.dtype)
    for d, t in st.degree_to_tensor.items():
        L = ctx.degree_to_layout[d]
        times = [a * ztime for a in L.edge_ampls]
        aligned = [st.msgs[p] for p in L.input_msgs_position]
        for m, p in zip(pass_msgs(t, aligned, times), L.output_msgs_position):
            new[p] = m
    return new


def apply_canonicalizers_with_extensions(t: np.ndarray, cans: list, couplings: list) -> np.ndarray:
    for C, c in zip(cans, couplings):                              # backends.py:416-432
        t = _extend_bond(t, 2, c, conj=False)
        t = _apply_first_bond(t, np.swapaxes(C, 1, 2))
    return t


def simple_update(ctx: OracleContext, ztime: float, st: OracleState) -> tuple[int, float]:
    ext = get_extended_msgs(ctx, ztime, st)                        # state.py:230-247
    lam, can = get_canonicalizers(ext, ctx.pinv_eps)
    dim, err = truncation_dim(lam, ctx.max_bond_dim, ctx.pinv_eps)
    st.lmbds = lam[:, :dim].astype(ctx.dtype)
    can = can[:, :, :dim]
    for d, L in ctx.degree_to_layout.items():
        aligned = [can[p] for p in L.input_msgs_position]
        couplings = [a * ztime for a in L.edge_ampls]
        st.degree_to_tensor[d] = apply_canonicalizers_with_extensions(st.degree_to_tensor[d], aligned, couplings)
    return dim, err


def apply_z_layer(ctx: OracleContext, ztime: float, st: OracleState) -> None:
    for d, t in st.degree_to_tensor.items():                       # state.py:142-150
        c = (ztime * ctx.degree_to_layout[d].node_ampls).astype(ctx.dtype)
        st.degree_to_tensor[d] = t * _bcast(np.cos(c), t.ndim) - 1j * _z_phys(t) * _bcast(np.sin(c), t.ndim)


def apply_x_layer(xtime: float, st: OracleState) -> None:
    for d, t in st.degree_to_tensor.items():                       # backends.py:506-507
        st.degree_to_tensor[d] = cos(xtime) * t - 1j * sin(xtime) * _x_phys(t)


def set_to_symmetric_gauge(ctx: OracleContext, st: OracleState) -> None:
    st.msgs = _msgs_from_lmbds(st.lmbds, ctx)                      # state.py:219-227
    for d, L in ctx.degree_to_layout.items():
        t = st.degree_to_tensor[d]
        for k, pos in enumerate(L.lmbds_position):                 # backends.py:450-462
            shape = [t.shape[0]] + [1] * (t.ndim - 1)
            shape[k + 2] = t.shape[k + 2]
            t = t * np.sqrt(st.lmbds[pos]).reshape(shape)
        norms = np.linalg.norm(t.reshape(t.shape[0], -1), axis=1)
        st.degree_to_tensor[d] = t / _bcast(norms, t.ndim)


def run_layer(ctx: OracleContext, xtime: float, ztime: float, st: OracleState) -> dict:
    """One annealing step (src/bqa/state.py:315-321); returns step statistics."""
    dim, err = simple_update(ctx, ztime, st)
    apply_z_layer(ctx, ztime, st)
    apply_x_layer(xtime, st)
    set_to_symmetric_gauge(ctx, st)
    sweeps = run_bp(ctx, st)
    return {"bond_dim": dim, "trunc_err": err, "sweeps": sweeps}


def get_density_matrices(ctx: OracleContext, st: OracleState) -> np.ndarray:
    """Per-node 2x2 marginals (src/bqa/state.py:77-94, backends.py:440-448).

    Degree-0 nodes (the reference asserts on them) get ``rho = psi psi^dagger``."""
    out = np.empty((ctx.nodes_number, 2, 2), ctx.dtype)
    for d, L in ctx.degree_to_layout.items():
        t = st.degree_to_tensor[d]
        tm = t
        for p in L.input_msgs_position:
            tm = _apply_first_bond(tm, st.msgs[p])
        B = t.shape[0]
        rho = tm.reshape(B, 2, -1) @ np.swapaxes(np.conj(t).reshape(B, 2, -1), 1, 2)
        out[L.node_ids] = _trace_normalize(rho)
    return out


def bloch_vectors(rho: np.ndarray) -> np.ndarray:
    """(n, 3) [x, y, z] from (n, 2, 2) densities (src/bqa/utils.py:23-27)."""
    x = (rho[:, 0, 1] + rho[:, 1, 0]).real
    y = (rho[:, 1, 0] - rho[:, 0, 1]).imag
    z = (rho[:, 0, 0] - rho[:, 1, 1]).real
    return np.stack([x, y, z], axis=1)


def edge_zz(ctx: OracleContext, st: OracleState) -> np.ndarray:
    """BP two-site estimate of <Z_u Z_v> for every undirected edge slot p < E/2.

    With ``P^u_s`` the open-bond block of u on its bond to v (``psplit_msgs``), and
    ``S = P_0 + P_1``, ``Z = P_0 - P_1``:
    ``<Z_u Z_v> = Re sum_ab Z^u[a,b] Z^v[a,b] / sum_ab S^u[a,b] S^v[a,b]``
    (ket bond index b and bra bond index a are shared by the two tensors)."""
    E = ctx.edges_number
    half = E // 2
    chi = st.bond_dim
    pm = np.zeros((E, 2, chi, chi), ctx.dtype)
    for d, t in st.degree_to_tensor.items():
        if d == 0:
            continue
        L = ctx.degree_to_layout[d]
        aligned = [st.msgs[p] for p in L.input_msgs_position]
        for ps, p in zip(psplit_msgs(t, aligned), L.output_msgs_position):
            pm[p] = ps
    S = pm[:, 0] + pm[:, 1]
    Z = pm[:, 0] - pm[:, 1]
    num = np.sum(Z[:half] * Z[half:], axis=(1, 2))
    den = np.sum(S[:half] * S[half:], axis=(1, 2))
    return (num / den).real


def energy(ctx: OracleContext, zz: np.ndarray, z: np.ndarray) -> float:
    """``sum_p J_p <Z Z>_p + sum_i h_i <Z_i>`` over undirected edges p."""
    half = ctx.edges_number // 2
    J = np.array([ctx.edge_to_ampl[e] for e in list(ctx.edge_to_ampl.keys())[:half]])
    h = np.array([ctx.node_to_ampl[v] for v in range(ctx.nodes_number)])
    return float(np.dot(J, zz) + np.dot(h, z))


def spin_energy(ctx: OracleContext, spins: np.ndarray) -> float:
    half = ctx.edges_number // 2
    keys = list(ctx.edge_to_ampl.keys())[:half]
    J = np.array([ctx.edge_to_ampl[e] for e in keys])
    a = np.array([e[0] for e in keys])
    b = np.array([e[1] for e in keys])
    h = np.array([ctx.node_to_ampl[v] for v in range(ctx.nodes_number)])
    return float(np.dot(J, spins[a] * spins[b]) + np.dot(h, spins))


def measure(ctx: OracleContext, st: OracleState) -> list:
    """Sequential most-polarised-first sampling (src/bqa/state.py:250-312)."""
    outcomes: dict = {}
    thr = ctx.measurement_threshold

    def project(node: int, outcome: int) -> None:
        outcomes[node] = 1 - 2 * outcome
        d, pos = ctx.path_to_tensors[node]
        t = st.degree_to_tensor[d]                                 # backends.py:730-734
        t[pos, 1 - outcome] = 0.0
        t /= np.linalg.norm(t)

    def ground_probs() -> dict:
        dens = get_density_matrices(ctx, st)
        return {v: float(dens[v, 0, 0].real) for v in range(ctx.nodes_number) if v not in outcomes}

    while len(outcomes) < ctx.nodes_number:
        probs = ground_probs()
        node, prob = max(probs.items(), key=lambda kv: abs(2 * kv[1] - 1))
        val = st.rng.uniform(0.0, 1.0)
        project(node, 0 if prob > val else 1)
        run_bp(ctx, st)
        probs = ground_probs()
        for v in [v for v, p in probs.items() if p > thr]:
            project(v, 0)
        for v in [v for v, p in probs.items() if p < 1.0 - thr]:
            project(v, 1)
        run_bp(ctx, st)
    return [outcomes[v] for v in range(len(outcomes))]


def run_qa(config: dict, dtype=np.complex128) -> list:
    """The reference ``run_qa`` result list (src/bqa/core.py:13-35)."""
    ctx = make_context(config, dtype)
    st = initialize_state(ctx)
    out = []
    for ins in ctx.instructions:
        if isinstance(ins, dict):
            run_layer(ctx, ins["xtime"], ins["ztime"], st)
        elif ins == cfg.MEASURE:
            out.append(["measurement_outcomes", measure(ctx, st)])
        elif ins == cfg.GET_BLOCH_VECTORS:
            out.append(["bloch_vectors", bloch_vectors(get_density_matrices(ctx, st)).tolist()])
        else:
            raise ValueError(f"Unknown instruction {ins}")
    return out
