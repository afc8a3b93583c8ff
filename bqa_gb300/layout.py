"""Degree-class compiler: graph -> integer batch maps (host side, vectorised).

Restates ``_make_degree_to_layout`` / ``_canonicalize_config``
(``src/bqa/config/config_canonicalization.py:62-131,182-249``) with numpy scans instead of
a per-node Python loop, so a 200k-node job compiles in milliseconds.

Conventions (identical to the reference, and checked bit-exact against its known-answer
test ``tests/test_config_to_context.py:68-119``):

* directed edge ``p`` (``0 <= p < E``) is the ``p``-th key of the analysed edge dict:
  ``p < E/2`` are the user's edges, ``p >= E/2`` their reversals in the same order;
  its BP message lives in message slot ``p`` and its bond spectrum in lambda slot
  ``p % (E/2)``;
* bond ``k`` of node ``v`` points to the ``k``-th directed edge (in slot order) that
  leaves ``v``;
* nodes are grouped by degree; classes are kept in order of first appearance over
  increasing node id (the reference's dict insertion order), nodes within a class in
  increasing id.

Per class the maps are ``(d, B)`` arrays (``k``-major, like the reference's lists of
``d`` tensors): ``input_msgs_position[k, i]`` = slot of the message ``nbr_k -> v``,
``output_msgs_position[k, i]`` = slot of ``v -> nbr_k``, ``lmbds_position[k, i]`` =
lambda slot of that edge; ``edge_ampls[k, i]`` its coupling ``J``; ``node_ampls[i]`` the
node field ``h``.  The device copies are node-major ``(B, d)`` int32 (one CTA reads its
node's ``d`` slots with one load).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import config as cfg


@dataclass
class DegreeClass:
    degree: int
    node_ids: np.ndarray              # (B,) int64
    input_msgs_position: np.ndarray   # (d, B) int64
    output_msgs_position: np.ndarray  # (d, B) int64
    lmbds_position: np.ndarray        # (d, B) int64
    node_ampls: np.ndarray            # (B,) float64
    edge_ampls: np.ndarray            # (d, B) float64

    @property
    def batch_size(self) -> int:
        return int(self.node_ids.shape[0])


@dataclass
class Context:
    """Everything a run needs that does not change while it runs (reference ``Context``)."""
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
    degree_to_layout: dict[int, DegreeClass]
    # per node: (degree, position inside its class)  (reference ``path_to_tensors``)
    node_degree: np.ndarray = field(repr=False)
    node_position: np.ndarray = field(repr=False)
    # per undirected edge p < E/2: endpoints and coupling
    edge_src: np.ndarray = field(repr=False)
    edge_dst: np.ndarray = field(repr=False)
    edge_ampl: np.ndarray = field(repr=False)
    node_ampl: np.ndarray = field(repr=False)   # (n,) field h of every node

    @property
    def lmbds_number(self) -> int:
        return self.edges_number // 2

    @property
    def msg_pos_to_lmbd_pos(self) -> np.ndarray:
        return np.arange(self.edges_number, dtype=np.int64) % self.lmbds_number

    @property
    def path_to_tensors(self) -> dict[int, tuple[int, int]]:
        return {int(v): (int(d), int(p)) for v, (d, p) in
                enumerate(zip(self.node_degree, self.node_position))}


def compile_layout(edge_list: np.ndarray, nodes_number: int):
    """Degree classes for ``E`` directed edges given as an ``(E, 2)`` array in slot order."""
    edges = np.asarray(edge_list, dtype=np.int64).reshape(-1, 2)
    E = edges.shape[0]
    half = E // 2
    src = edges[:, 0]
    deg = np.bincount(src, minlength=nodes_number).astype(np.int64)
    order = np.argsort(src, kind="stable")            # slots grouped by source, slot order inside
    start = np.zeros(nodes_number, dtype=np.int64)
    np.cumsum(deg[:-1], out=start[1:])
    # classes in order of first appearance over node ids
    uniq, first = np.unique(deg, return_index=True)
    class_degrees = [int(d) for d in uniq[np.argsort(first)]]
    classes = {}
    node_position = np.empty(nodes_number, dtype=np.int64)
    for d in class_degrees:
        nodes = np.flatnonzero(deg == d)
        node_position[nodes] = np.arange(nodes.shape[0])
        if d > 0:
            slots = order[start[nodes][:, None] + np.arange(d)[None, :]].T   # (d, B) v -> nbr_k
        else:
            slots = np.zeros((0, nodes.shape[0]), dtype=np.int64)
        classes[d] = (nodes, slots)
    return classes, deg, node_position


def compile_layout_device(edge_list: np.ndarray, nodes_number: int, device=None, max_degree: int = 255):
    """``compile_layout`` computed on the GPU (``bqa_layout_degrees`` + ``bqa_layout_class``):
    degree histogram and slot grouping by atomics, per-node slot sort, per-degree stream
    compaction by a single-CTA scan.  Returns the same ``(classes, deg, node_position)``,
    bit for bit, copied back to host memory."""
    import torch
    from . import _lib
    lib = _lib.load()
    dev = torch.device(device if device is not None else "cuda")
    edges = np.asarray(edge_list, dtype=np.int64).reshape(-1, 2)
    E, n = edges.shape[0], int(nodes_number)
    if E >= 2 ** 31 or n >= 2 ** 31:
        raise ValueError("the device layout compiler takes fewer than 2^31 edges and nodes")
    d_edges = torch.as_tensor(edges.astype(np.int32), device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    deg, start, fill, position = (torch.empty(n, **i32) for _ in range(4))
    order = torch.empty(E, **i32)
    first = torch.empty(max_degree + 1, **i32)
    count = torch.empty(max_degree + 1, **i32)
    status = torch.zeros(1, **i32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    p = lambda t: t.data_ptr()
    lib.call("bqa_layout_degrees", p(d_edges), E, n, max_degree, p(deg), p(start), p(order), p(fill), p(first),
             p(count), p(status), stream)
    st = int(status.cpu()[0])
    if st & _lib.BQA_STATUS_LAYOUT_EDGE:
        raise ValueError("edge list has an endpoint outside [0, n), a self-loop, or a slot whose reversal "
                         "is not at slot + E/2")
    if st & _lib.BQA_STATUS_LAYOUT_DEGREE:
        raise ValueError(f"a node has degree above {max_degree}")
    first_h, count_h = first.cpu().numpy(), count.cpu().numpy()
    degrees = sorted((d for d in range(max_degree + 1) if count_h[d] > 0), key=lambda d: int(first_h[d]))
    out = {}
    for d in degrees:
        B = int(count_h[d])
        node_ids = torch.empty(B, **i32)
        slots = torch.empty(B * d, **i32) if d > 0 else None
        lib.call("bqa_layout_class", d, B, p(deg), p(start), p(order), n, E, None, None, p(node_ids), p(position),
                 None, p(slots) if slots is not None else None, None, None, None, stream)
        out[d] = (node_ids, slots)
    classes = {}
    for d, (node_ids, slots) in out.items():
        B = node_ids.shape[0]
        sl = (slots.view(B, d).T.cpu().numpy().astype(np.int64) if d > 0
              else np.zeros((0, B), dtype=np.int64))
        classes[d] = (node_ids.cpu().numpy().astype(np.int64), sl)
    return classes, deg.cpu().numpy().astype(np.int64), position.cpu().numpy().astype(np.int64)


# directed-edge count from which build_context compiles on the device when given one
DEVICE_LAYOUT_MIN_EDGES = 1 << 16


def build_context(config: dict, layout_device=None) -> Context:
    """Analyse a user config and compile its degree classes (reference ``config_to_context``).
    With ``layout_device`` set, graphs of at least ``DEVICE_LAYOUT_MIN_EDGES`` directed edges
    are compiled by the device layout compiler (identical maps)."""
    c = cfg.analyse_config(config, edge_arrays=True)
    edge_list, ampl = c[cfg.EDGES_KEY]
    if edge_list.shape[0] == 0:
        raise cfg.ConfigSyntaxError("Invalid config") from cfg.ConfigSyntaxError(
            "`edges` must hold at least one edge")
    E = edge_list.shape[0]
    half = E // 2
    node_ids, node_fields = c[cfg.NODES_KEY]
    n = 1 + max(int(node_ids.max()) if node_ids.size else -1, int(edge_list.max()))
    node_ampl = np.full(n, c[cfg.DEFAULT_FIELD_KEY], dtype=np.float64)
    node_ampl[node_ids] = node_fields
    if layout_device is not None and E >= DEVICE_LAYOUT_MIN_EDGES:
        classes, deg, node_position = compile_layout_device(edge_list, n, layout_device)
    else:
        classes, deg, node_position = compile_layout(edge_list, n)
    layouts = {}
    for d, (nodes, slots) in classes.items():
        rev = (slots + half) % E if d > 0 else slots
        layouts[d] = DegreeClass(
            degree=d,
            node_ids=nodes,
            input_msgs_position=rev,
            output_msgs_position=slots,
            lmbds_position=slots % half if d > 0 else slots,
            node_ampls=node_ampl[nodes],
            edge_ampls=ampl[slots] if d > 0 else np.zeros((0, nodes.shape[0])),
        )
    return Context(
        nodes_number=n,
        edges_number=E,
        max_bond_dim=c[cfg.MAX_BOND_DIM_KEY],
        max_bp_iters_number=c[cfg.MAX_BP_ITER_NUMBER_KEY],
        bp_eps=c[cfg.BP_EPS_KEY],
        pinv_eps=c[cfg.PINV_EPS_KEY],
        measurement_threshold=c[cfg.MEASUREMENT_THRESHOLD_KEY],
        damping=c[cfg.DAMPING_KEY],
        seed=c[cfg.SEED_KEY],
        instructions=cfg.canonicalize_schedule(c[cfg.SCHEDULE_KEY]),
        degree_to_layout=layouts,
        node_degree=deg,
        node_position=node_position,
        edge_src=edge_list[:half, 0].copy(),
        edge_dst=edge_list[:half, 1].copy(),
        edge_ampl=ampl[:half].copy(),
        node_ampl=node_ampl,
    )
