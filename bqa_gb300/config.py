"""Annealing-job config analysis for the GB300 backend.

The job description is the reference's dict DSL, unchanged, so a config written for
``bqa.run_qa`` runs here as is.  This module restates its validation, defaults and
schedule expansion:

* keys, defaults and value checks: ``src/bqa/config/config_syntax.py:15-191`` and
  ``src/bqa/config/utils.py:1-86``;
* schedule desugaring and expansion into per-step ``{"xtime", "ztime"}`` instructions:
  ``src/bqa/config/schedule_syntax.py:39-169`` and
  ``src/bqa/config/schedule_canonicalization.py:1-33``.

The one behaviour that the device layout depends on is the EDGE ORDER: every undirected
edge ``(a, b)`` is entered once as a forward edge, in the order the user listed it, and
the reversed edges ``(b, a)`` follow in the same order (``config_syntax.py:118-154``).
Message slot ``p`` is the ``p``-th edge of that order.

The only deliberate difference: the backend key defaults to ``"gb300"`` and only the
backends registered in :data:`BACKENDS` are accepted.
"""
from __future__ import annotations

import logging
from itertools import chain
from math import isclose
from typing import NamedTuple

import numpy as np

log = logging.getLogger(__name__)


class ConfigSyntaxError(ValueError):
    """Invalid job config (same class name and base as the reference's)."""


# keys (reference config_syntax.py:17-39, schedule_syntax.py:21-37)
NODES_KEY = "nodes"
EDGES_KEY = "edges"
DEFAULT_FIELD_KEY = "default_field"
SCHEDULE_KEY = "schedule"
MAX_BOND_DIM_KEY = "max_bond_dim"
MAX_BP_ITER_NUMBER_KEY = "max_bp_iter_number"
SEED_KEY = "seed"
BP_EPS_KEY = "bp_eps"
PINV_EPS_KEY = "pinv_eps"
MEASUREMENT_THRESHOLD_KEY = "measurement_threshold"
DAMPING_KEY = "damping"
BACKEND_KEY = "backend"

FINAL_MIXING_KEY = "final_mixing"
INITIAL_MIXING_KEY = "initial_mixing"
STARTING_MIXING_KEY = "starting_mixing"
TYPE_KEY = "type"
TOTAL_TIME_KEY = "total_time"
ACTIONS_KEY = "actions"
WEIGHT_KEY = "weight"
STEPS_NUMBER_KEY = "steps_number"

GET_BLOCH_VECTORS = "get_bloch_vectors"
MEASURE = "measure"
REAL_TIME_EV_TYPE = "real_time_evolution"
IMAG_TIME_EV_TYPE = "imag_time_evolution"
SIMPLE_ACTION_TYPES = frozenset({MEASURE, GET_BLOCH_VECTORS})
COMPLEX_ACTION_TYPES = frozenset({REAL_TIME_EV_TYPE, IMAG_TIME_EV_TYPE})
ACTION_TYPES = SIMPLE_ACTION_TYPES | COMPLEX_ACTION_TYPES

# backends this package executes; the reference keeps the same registry keyed by name
# (src/bqa/backends.py:26) and validates the key against it (config_syntax.py:63-70)
BACKENDS = ("gb300",)

# defaults (reference config_syntax.py:43-61, schedule_syntax.py:41-73)
DEFAULTS = {
    NODES_KEY: {},
    MAX_BOND_DIM_KEY: 4,
    MAX_BP_ITER_NUMBER_KEY: 75,
    BP_EPS_KEY: 1e-6,
    PINV_EPS_KEY: 1e-6,
    BACKEND_KEY: "gb300",
    DEFAULT_FIELD_KEY: 0.0,
    MEASUREMENT_THRESHOLD_KEY: 0.95,
    SEED_KEY: 42,
    DAMPING_KEY: 0.0,
}
DEFAULT_EVOLUTION = {
    TYPE_KEY: REAL_TIME_EV_TYPE,
    WEIGHT_KEY: 1.0,
    STEPS_NUMBER_KEY: 100,
    FINAL_MIXING_KEY: 0.0,
}
DEFAULT_SCHEDULE = {
    TOTAL_TIME_KEY: 10.0,
    STARTING_MIXING_KEY: 1.0,
    ACTIONS_KEY: [DEFAULT_EVOLUTION, GET_BLOCH_VECTORS],
}


def _take(dct, key, default, where):
    """Value of ``key`` or ``default`` with a warning when absent (or None)."""
    val = dct.get(key)
    if val is None:
        log.warning(f"`{key}` field is missing in {where}, set to default {default}")
        return default
    return val


def _require(dct, key, where):
    val = dct.get(key)
    if val is None:
        raise ConfigSyntaxError(f"`{key}` field is missing in {where}")
    return val


def _is_num(x) -> bool:
    return isinstance(x, (float, int))


def _check(pred: bool, value, what: str):
    if not pred:
        raise ConfigSyntaxError(f"Invalid value {value}, {what}")


def _number(x) -> float:
    _check(_is_num(x), x, "must be a `float` or `int` number")
    return float(x)


def _non_neg_number(x) -> float:
    _check(_is_num(x) and x >= 0.0, x, "must be a non-negative `float` or `int` number")
    return float(x)


def _unit_number(x) -> float:
    _check(_is_num(x) and 0.0 <= x <= 1.0, x, "must be a `float` or `int` number from [0, 1]")
    return float(x)


def _half_unit_number(x) -> float:
    _check(_is_num(x) and 0.5 <= x <= 1.0, x, "must be a `float` or `int` number from [0.5, 1]")
    return float(x)


def _non_neg_int(x) -> int:
    _check(isinstance(x, int) and x >= 0, x, "must be a non-negative `int`")
    return x


def _positive_int(x) -> int:
    _check(isinstance(x, int) and x > 0, x, "must be a positive `int`")
    return x


def _backend(name):
    if not isinstance(name, str):
        raise ConfigSyntaxError(f"Invalid backend \"{name}\"")
    if name not in BACKENDS:
        raise ConfigSyntaxError(f"Unknown backend \"{name}\", available backends {list(BACKENDS)}")
    return name


def _nodes(nodes) -> dict[int, float]:
    if not isinstance(nodes, (tuple, list, dict)):
        raise ConfigSyntaxError(f"Invalid nodes {nodes}")
    out: dict[int, float] = {}
    pairs = nodes.items() if isinstance(nodes, dict) else nodes
    try:
        for node in pairs:
            if not (isinstance(node, (tuple, list)) and len(node) == 2):
                raise ConfigSyntaxError(f"Invalid node {node}")
            try:
                node_id = _non_neg_int(node[0])
                field = _number(node[1])
                if node_id in out:
                    raise ConfigSyntaxError(f"Duplicated node ID {node_id}")
            except ConfigSyntaxError as e:
                raise ConfigSyntaxError(f"Invalid node {node}") from e
            out[node_id] = field
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError(f"Invalid nodes {nodes}") from e
    return out


def _edge_id(edge_id) -> tuple[int, int]:
    if not (isinstance(edge_id, (list, tuple)) and len(edge_id) == 2):
        raise ConfigSyntaxError(f"Invalid edge ID {edge_id}")
    try:
        lhs = _non_neg_int(edge_id[0])
        rhs = _non_neg_int(edge_id[1])
        if lhs == rhs:
            raise ConfigSyntaxError(
                f"LHS and RHS of the edge ID must not be equal, got edge ID {edge_id}")
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError(f"Invalid edge ID {edge_id}") from e
    return lhs, rhs


def _edges(edges) -> dict[tuple[int, int], float]:
    """Forward edges in user order, then every edge reversed in the same order."""
    if not isinstance(edges, (dict, tuple, list)):
        raise ConfigSyntaxError(f"Invalid edges {edges}")
    fwd: dict[tuple[int, int], float] = {}
    seen: set[tuple[int, int]] = set()
    pairs = edges.items() if isinstance(edges, dict) else edges
    try:
        for edge in pairs:
            if not (isinstance(edge, (tuple, list)) and len(edge) == 2):
                raise ConfigSyntaxError(f"Invalid edge {edge}")
            try:
                lhs, rhs = _edge_id(edge[0])
                coupling = _number(edge[1])
                if (lhs, rhs) in seen or (rhs, lhs) in seen:
                    raise ConfigSyntaxError(f"Duplicated edge ID {(lhs, rhs)}, {(rhs, lhs)}")
            except ConfigSyntaxError as e:
                raise ConfigSyntaxError(f"Invalid edge {edge}") from e
            seen.add((lhs, rhs))
            fwd[(lhs, rhs)] = coupling
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError(f"Invalid edges {edges}") from e
    both = dict(fwd)
    for (lhs, rhs), coupling in fwd.items():
        both[(rhs, lhs)] = coupling
    return both


def _desugar_actions(actions, starting_mixing):
    """Give every action an explicit initial/final mixing (schedule_syntax.py:283-313)."""
    mixing = starting_mixing
    for action in actions:
        if isinstance(action, dict):
            act = dict(action)
            if INITIAL_MIXING_KEY in act:
                raise ConfigSyntaxError(
                    f"`{INITIAL_MIXING_KEY}` must not be present in the action {act}, "
                    "it is infered automatically")
            act[INITIAL_MIXING_KEY] = mixing
            if FINAL_MIXING_KEY in act:
                mixing = act[FINAL_MIXING_KEY]
            else:
                act[FINAL_MIXING_KEY] = mixing
            yield act
        elif isinstance(action, str):
            yield {TYPE_KEY: action, WEIGHT_KEY: 0, INITIAL_MIXING_KEY: mixing,
                   FINAL_MIXING_KEY: mixing, STEPS_NUMBER_KEY: 1}
        else:
            raise TypeError(f"Invalid type {type(action)} of the action {action}")


def _analyse_actions(actions, starting_mixing):
    if not isinstance(actions, (list, tuple)):
        raise ConfigSyntaxError(
            f"Actions must be either a list or a tuple, got {actions} of type {type(actions)}")
    try:
        out = []
        for act in _desugar_actions(actions, starting_mixing):
            kind = _take(act, TYPE_KEY, REAL_TIME_EV_TYPE, "action")
            if kind not in ACTION_TYPES:
                raise ConfigSyntaxError(f"Invalid action type {kind} in action {act}")
            out.append({
                TYPE_KEY: kind,
                WEIGHT_KEY: _unit_number(_require(act, WEIGHT_KEY, "action")),
                STEPS_NUMBER_KEY: _positive_int(_take(act, STEPS_NUMBER_KEY, 100, "action")),
                INITIAL_MIXING_KEY: _unit_number(act[INITIAL_MIXING_KEY]),
                FINAL_MIXING_KEY: _unit_number(act[FINAL_MIXING_KEY]),
            })
        total = sum(a[WEIGHT_KEY] for a in out)
        if not isclose(total, 1.0):
            raise ConfigSyntaxError(
                f"`{WEIGHT_KEY}` fields must sum into 1. in actions {out}, but now it sums into {total}")
        return out
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError(f"Invalid actions {actions}") from e


def _schedule(schedule):
    if not isinstance(schedule, dict):
        raise ConfigSyntaxError(f"Schedule must be a dict, got {schedule} of type {type(schedule)}")
    try:
        total_time = _non_neg_number(_take(schedule, TOTAL_TIME_KEY, 10.0, "schedule"))
        mixing = _unit_number(_take(schedule, STARTING_MIXING_KEY, 1.0, "schedule"))
        actions = _analyse_actions(_take(schedule, ACTIONS_KEY, DEFAULT_SCHEDULE[ACTIONS_KEY], "schedule"),
                                   mixing)
        return {TOTAL_TIME_KEY: total_time, ACTIONS_KEY: actions}
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError(f"Invalid schedule {schedule}") from e


class EdgeArrays(NamedTuple):
    """Analysed edges as arrays: ``edges[p]`` = (src, dst) of directed edge (message slot)
    ``p`` -- the user's edges in order, then their reversals -- and ``ampl[p]`` its coupling."""
    edges: np.ndarray   # (E, 2) int64
    ampl: np.ndarray    # (E,) float64


# edge collections from this size are first offered to the vectorised acceptance test
FAST_EDGES_MIN = 1024


def _all_subclasses(kinds, base) -> bool:
    return all(issubclass(k, base) for k in kinds)


def _edges_fast(edges) -> EdgeArrays | None:
    """Vectorised form of ``_edges`` for large edge collections: the same acceptance rules
    (pairs of a 2-sequence of non-negative ``int`` ends that differ and a ``float``/``int``
    coupling, no edge given twice in either orientation), checked on whole arrays.  Returns
    None when any rule might fail; ``_edges`` then walks the input and raises the exact error."""
    if isinstance(edges, dict):
        ids, vals = list(edges.keys()), list(edges.values())
    elif isinstance(edges, (list, tuple)):
        if not _all_subclasses(set(map(type, edges)), (list, tuple)) or set(map(len, edges)) != {2}:
            return None
        ids, vals = [e[0] for e in edges], [e[1] for e in edges]
    else:
        return None
    if not ids:
        return None
    if not _all_subclasses(set(map(type, ids)), (list, tuple)) or set(map(len, ids)) != {2}:
        return None
    if not _all_subclasses(set(map(type, chain.from_iterable(ids))), int):
        return None
    if not _all_subclasses(set(map(type, vals)), (int, float)):
        return None
    try:
        arr = np.array(ids, dtype=np.int64)
        ampl = np.array(vals, dtype=np.float64)
    except (OverflowError, ValueError, TypeError):
        return None
    if arr.ndim != 2 or arr.shape[1] != 2 or (arr < 0).any() or (arr[:, 0] == arr[:, 1]).any():
        return None
    lo, hi = np.minimum(arr[:, 0], arr[:, 1]), np.maximum(arr[:, 0], arr[:, 1])
    if int(hi.max()) >= 2 ** 31:
        return None
    key = np.sort(lo * (2 ** 31) + hi)
    if (key[1:] == key[:-1]).any():
        return None
    return EdgeArrays(np.concatenate([arr, arr[:, ::-1]]), np.concatenate([ampl, ampl]))


class NodeArrays(NamedTuple):
    """Analysed node fields as arrays, in the user's order."""
    ids: np.ndarray     # (m,) int64
    fields: np.ndarray  # (m,) float64


def _nodes_fast(nodes) -> NodeArrays | None:
    """Vectorised form of ``_nodes`` (same acceptance rules: pairs of a non-negative ``int`` id
    and a ``float``/``int`` field, no id twice); None when any rule might fail."""
    if isinstance(nodes, dict):
        ids, vals = list(nodes.keys()), list(nodes.values())
    elif isinstance(nodes, (list, tuple)):
        if not _all_subclasses(set(map(type, nodes)), (list, tuple)) or set(map(len, nodes)) != {2}:
            return None
        ids, vals = [e[0] for e in nodes], [e[1] for e in nodes]
    else:
        return None
    if not ids or not _all_subclasses(set(map(type, ids)), int) \
            or not _all_subclasses(set(map(type, vals)), (int, float)):
        return None
    try:
        arr = np.array(ids, dtype=np.int64)
        fields = np.array(vals, dtype=np.float64)
    except (OverflowError, ValueError, TypeError):
        return None
    if (arr < 0).any():
        return None
    if not isinstance(nodes, dict):   # dict keys are distinct already
        srt = np.sort(arr)
        if (srt[1:] == srt[:-1]).any():
            return None
    return NodeArrays(arr, fields)


def analyse_config(config, edge_arrays: bool = False) -> dict:
    """Validated config with defaults applied (reference ``_analyse_config``).  With
    ``edge_arrays`` the edges and nodes come back as ``EdgeArrays`` and ``NodeArrays``
    instead of dicts (large collections are then validated by whole-array checks)."""
    if not isinstance(config, dict):
        raise ConfigSyntaxError(f"Config must be a dict, but got type {type(config)}")
    try:
        w = "config"
        nodes = _take(config, NODES_KEY, DEFAULTS[NODES_KEY], w)
        edges = _require(config, EDGES_KEY, w)
        schedule = _take(config, SCHEDULE_KEY, DEFAULT_SCHEDULE, w)
        out = {
            MAX_BOND_DIM_KEY: _take(config, MAX_BOND_DIM_KEY, DEFAULTS[MAX_BOND_DIM_KEY], w),
            MAX_BP_ITER_NUMBER_KEY: _take(config, MAX_BP_ITER_NUMBER_KEY, DEFAULTS[MAX_BP_ITER_NUMBER_KEY], w),
            BP_EPS_KEY: _take(config, BP_EPS_KEY, DEFAULTS[BP_EPS_KEY], w),
            PINV_EPS_KEY: _take(config, PINV_EPS_KEY, DEFAULTS[PINV_EPS_KEY], w),
            BACKEND_KEY: _take(config, BACKEND_KEY, DEFAULTS[BACKEND_KEY], w),
            DEFAULT_FIELD_KEY: _take(config, DEFAULT_FIELD_KEY, DEFAULTS[DEFAULT_FIELD_KEY], w),
            MEASUREMENT_THRESHOLD_KEY: _take(config, MEASUREMENT_THRESHOLD_KEY,
                                             DEFAULTS[MEASUREMENT_THRESHOLD_KEY], w),
            SEED_KEY: _take(config, SEED_KEY, DEFAULTS[SEED_KEY], w),
            DAMPING_KEY: _take(config, DAMPING_KEY, DEFAULTS[DAMPING_KEY], w),
        }
        nodes_out = None
        if edge_arrays and isinstance(nodes, (dict, list, tuple)) and len(nodes) >= FAST_EDGES_MIN:
            nodes_out = _nodes_fast(nodes)
        if nodes_out is None:
            nodes_out = _nodes(nodes)
            if edge_arrays:
                nodes_out = NodeArrays(np.array(list(nodes_out.keys()), dtype=np.int64),
                                       np.array(list(nodes_out.values()), dtype=np.float64))
        if edge_arrays:
            fast = _edges_fast(edges) if isinstance(edges, (dict, list, tuple)) and len(edges) >= FAST_EDGES_MIN \
                else None
            if fast is None:
                both = _edges(edges)
                fast = EdgeArrays(np.array(list(both.keys()), dtype=np.int64).reshape(-1, 2),
                                  np.array(list(both.values()), dtype=np.float64))
            edges_out = fast
        else:
            edges_out = _edges(edges)
        return {
            NODES_KEY: nodes_out,
            EDGES_KEY: edges_out,
            DEFAULT_FIELD_KEY: _number(out[DEFAULT_FIELD_KEY]),
            SCHEDULE_KEY: _schedule(schedule),
            MAX_BOND_DIM_KEY: _positive_int(out[MAX_BOND_DIM_KEY]),
            MAX_BP_ITER_NUMBER_KEY: _non_neg_int(out[MAX_BP_ITER_NUMBER_KEY]),
            SEED_KEY: _non_neg_int(out[SEED_KEY]),
            BP_EPS_KEY: _non_neg_number(out[BP_EPS_KEY]),
            PINV_EPS_KEY: _unit_number(out[PINV_EPS_KEY]),
            MEASUREMENT_THRESHOLD_KEY: _half_unit_number(out[MEASUREMENT_THRESHOLD_KEY]),
            DAMPING_KEY: _unit_number(out[DAMPING_KEY]),
            BACKEND_KEY: _backend(out[BACKEND_KEY]),
        }
    except ConfigSyntaxError as e:
        raise ConfigSyntaxError("Invalid config") from e


def canonicalize_schedule(schedule: dict) -> list:
    """Expand an analysed schedule into the instruction list.

    Evolution actions become ``steps_number`` dicts ``{"type", "xtime", "ztime"}`` with the
    mixing ``p`` interpolated linearly (endpoint excluded): ``xtime = p*dt``,
    ``ztime = (1-p)*dt``, ``dt = total_time*weight/steps_number``; the simple actions
    ``"measure"`` and ``"get_bloch_vectors"`` stay strings
    (reference ``schedule_canonicalization.py:4-33``).
    """
    total_time = schedule[TOTAL_TIME_KEY]
    out: list = []
    for act in schedule[ACTIONS_KEY]:
        kind = act[TYPE_KEY]
        if kind in COMPLEX_ACTION_TYPES:
            steps = act[STEPS_NUMBER_KEY]
            dt = total_time * act[WEIGHT_KEY] / steps
            start, end = act[INITIAL_MIXING_KEY], act[FINAL_MIXING_KEY]
            delta = (end - start) / steps
            for k in range(steps):
                p = start + k * delta
                out.append({"type": kind, "xtime": p * dt, "ztime": (1.0 - p) * dt})
        else:
            out.append(kind)
    return out
