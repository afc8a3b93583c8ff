"""Degree-class compiler and config DSL: bit-exact against the reference's known answers.

The expected maps are the reference's own known-answer test
(``tests/test_config_to_context.py:35-165``); the product compiler (vectorised) and the
oracle's per-node loop restatement must both reproduce them, and agree with each other on
every golden case.
"""
from itertools import chain
from math import isclose
from operator import sub

import numpy as np
import pytest

from bqa_gb300 import config as cfg
from bqa_gb300.layout import build_context
from oracle import bqa_oracle as orc
from tests import golden_cases as gc

KNOWN_CONFIG = {
    "edges": {(0, 2): 1.0, (1, 0): -1, (3, 0): 0.1, (2, 4): 1.1, (1, 4): 0, (3, 1): 1},
    "nodes": {2: 1, 6: -1.1},
    "default_field": -0.5,
    "schedule": {
        "starting_mixing": 0.8,
        "total_time": 5,
        "actions": [
            {"weight": 0.4, "final_mixing": 0.3, "steps_number": 8},
            "measure",
            {"type": "imag_time_evolution", "weight": 0.6, "final_mixing": 0.11, "steps_number": 10},
            "get_bloch_vectors",
        ],
    },
    "damping": 0.3,
}

# (node_ids, input, output, lmbds, node_ampls, edge_ampls) per degree, from the reference test
KNOWN_LAYOUT = {
    0: ([5, 6], [], [], [], [-0.5, -1.1], []),
    2: ([2, 3, 4], [[9, 8, 3], [0, 11, 4]], [[3, 2, 9], [6, 5, 10]], [[3, 2, 3], [0, 5, 4]],
        [1.0, -0.5, -0.5], [[1.1, 0.1, 1.1], [1.0, 1.0, 0.0]]),
    3: ([0, 1], [[6, 7], [1, 10], [2, 5]], [[0, 1], [7, 4], [8, 11]], [[0, 1], [1, 4], [2, 5]],
        [-0.5, -0.5], [[1.0, -1.0], [-1.0, 0.0], [0.1, 1.0]]),
}


def _check_known(layouts):
    assert sorted(layouts.keys()) == [0, 2, 3]
    for d, (ids, inp, out, lam, na, ea) in KNOWN_LAYOUT.items():
        L = layouts[d]
        assert np.array_equal(np.asarray(L.node_ids), ids)
        for got, want in ((L.input_msgs_position, inp), (L.output_msgs_position, out),
                          (L.lmbds_position, lam)):
            assert len(got) == len(want)
            for g, w in zip(got, want):
                assert np.array_equal(np.asarray(g), w)
        assert np.allclose(np.asarray(L.node_ampls), na)
        for g, w in zip(L.edge_ampls, ea):
            assert np.allclose(np.asarray(g), w)


def test_known_answer_product_layout():
    ctx = build_context(dict(KNOWN_CONFIG))
    assert ctx.edges_number == 12
    assert ctx.nodes_number == 7
    assert ctx.max_bp_iters_number == 75
    assert isclose(ctx.bp_eps, 1e-6)
    assert isclose(ctx.damping, 0.3)
    assert ctx.max_bond_dim == 4
    _check_known(ctx.degree_to_layout)
    # class order = first appearance over node ids (reference dict insertion order)
    assert list(ctx.degree_to_layout.keys()) == [3, 2, 0]
    for node_id, (degree, pos) in ctx.path_to_tensors.items():
        assert ctx.degree_to_layout[degree].node_ids[pos] == node_id


def test_known_answer_oracle_layout():
    _check_known(orc.make_context(dict(KNOWN_CONFIG)).degree_to_layout)


def test_schedule_expansion_known_answer():
    ins = build_context(dict(KNOWN_CONFIG)).instructions
    assert ins[8] == "measure" and ins[-1] == "get_bloch_vectors"
    steps = [i for i in ins if isinstance(i, dict)]
    tot = lambda xs: sum(i["xtime"] + i["ztime"] for i in xs)
    assert isclose(tot(steps), 5.0)
    assert isclose(tot(ins[:8]), 5.0 * 0.4)
    assert isclose(tot([i for i in ins[8:] if isinstance(i, dict)]), 5.0 * 0.6)
    mix = [i["xtime"] / (i["xtime"] + i["ztime"]) for i in steps]
    first, second = mix[:8], mix[8:]
    assert isclose(first[0], 0.8) and isclose(second[0], 0.3)
    d1 = list(map(sub, chain(first[1:], [second[0]]), first))
    d2 = list(map(sub, chain(second[1:], [0.11]), second))
    assert all(isclose(x, d1[0]) for x in d1)
    assert all(isclose(x, d2[0]) for x in d2)
    assert steps[9]["type"] == "imag_time_evolution"


@pytest.mark.parametrize("name", gc.case_names())
def test_product_layout_matches_oracle_loop(name):
    conf = gc.config(name)
    ctx = build_context(dict(conf))
    octx = orc.make_context(dict(conf))
    assert list(ctx.degree_to_layout.keys()) == list(octx.degree_to_layout.keys())
    for d, L in ctx.degree_to_layout.items():
        O = octx.degree_to_layout[d]
        assert np.array_equal(L.node_ids, O.node_ids)
        for a, b in ((L.input_msgs_position, O.input_msgs_position),
                     (L.output_msgs_position, O.output_msgs_position),
                     (L.lmbds_position, O.lmbds_position)):
            assert np.array_equal(np.asarray(a).reshape(d, -1), np.asarray(b).reshape(d, -1))
        assert np.array_equal(L.node_ampls, O.node_ampls)
        assert np.array_equal(np.asarray(L.edge_ampls).reshape(d, -1), np.asarray(O.edge_ampls).reshape(d, -1))
    assert ctx.instructions == octx.instructions


@pytest.mark.parametrize("bad, msg", [
    ([], "Config must be a dict"),
    ({"nodes": {}}, "`edges` field is missing"),
    ({"edges": {(0, 0): 1.0}}, "must not be equal"),
    ({"edges": {(0, 1): 1.0, (1, 0): 2.0}}, "Duplicated edge"),
    ({"edges": {(0, 1): 1.0}, "nodes": [(0, 1.0), (0, 2.0)]}, "Duplicated node"),
    ({"edges": {(0, 1): 1.0}, "max_bond_dim": 0}, "positive"),
    ({"edges": {(0, 1): 1.0}, "pinv_eps": 2.0}, "[0, 1]"),
    ({"edges": {(0, 1): 1.0}, "measurement_threshold": 0.2}, "[0.5, 1]"),
    ({"edges": {(0, 1): 1.0}, "backend": "cupy"}, "Unknown backend"),
    ({"edges": {(0, 1): 1.0}, "schedule": {"actions": [{"weight": 0.5}]}}, "sum into 1"),
    ({"edges": {(0, 1): 1.0}, "schedule": {"actions": [{"weight": 1.0, "initial_mixing": 0.1}]}}, "infered"),
    ({"edges": {(0, 1): 1.0}, "schedule": {"actions": [{"weight": 1.0, "type": "bogus"}]}}, "Invalid action type"),
    ({"edges": {}}, "at least one edge"),
])
def test_config_errors(bad, msg):
    with pytest.raises(cfg.ConfigSyntaxError) as ei:
        build_context(bad)
    chain_msgs = []
    e = ei.value
    while e is not None:
        chain_msgs.append(str(e))
        e = e.__cause__
    assert any(msg in m for m in chain_msgs), chain_msgs


def test_defaults_and_instruction_dicts():
    ctx = build_context({"edges": {(0, 1): 1.0, (1, 2): -1.0}})
    assert ctx.max_bond_dim == 4 and ctx.max_bp_iters_number == 75 and ctx.seed == 42
    assert ctx.measurement_threshold == 0.95 and ctx.pinv_eps == 1e-6
    assert len(ctx.instructions) == 101 and ctx.instructions[-1] == "get_bloch_vectors"
    assert ctx.instructions[0] == {"type": "real_time_evolution", "xtime": 0.1, "ztime": 0.0}
