"""Whole-array validation of large edge/node collections gives what the element-wise
validation gives: the same arrays for valid inputs, the same exception for invalid ones."""
import numpy as np
import pytest

from bqa_gb300 import config as cfg, instances
from bqa_gb300.layout import build_context


def _slow_arrays(c):
    e = c[cfg.EDGES_KEY]
    n = c[cfg.NODES_KEY]
    return (np.array(list(e.keys()), dtype=np.int64), np.array(list(e.values())),
            np.array(list(n.keys()), dtype=np.int64), np.array(list(n.values())))


def _job(n=3000, form="dict"):
    conf = instances.headline_gpu_job(n=n, steps=3)
    if form == "list":   # JSON form: [[[u, v], J], ...], [[i, h], ...]
        conf = dict(conf, edges=[[list(k), v] for k, v in conf["edges"].items()],
                    nodes=[[k, v] for k, v in conf["nodes"].items()])
    return conf


@pytest.mark.parametrize("form", ["dict", "list"])
def test_fast_equals_slow(form):
    conf = _job(form=form)
    assert cfg._edges_fast(conf["edges"]) is not None
    fast = cfg.analyse_config(conf, edge_arrays=True)
    slow = cfg.analyse_config(conf)
    se, sa, sn, sf = _slow_arrays(slow)
    assert np.array_equal(fast[cfg.EDGES_KEY].edges, se)
    assert np.array_equal(fast[cfg.EDGES_KEY].ampl, sa)
    assert np.array_equal(fast[cfg.NODES_KEY].ids, sn)
    assert np.array_equal(fast[cfg.NODES_KEY].fields, sf)
    for k in slow:
        if k not in (cfg.EDGES_KEY, cfg.NODES_KEY):
            assert fast[k] == slow[k]


def _mutate(edges, i, new):
    items = list(edges.items())
    items[i] = new
    return items


@pytest.mark.parametrize("case", ["dup", "dup_reversed", "neg", "self", "np_int", "str_coupling", "short"])
def test_invalid_inputs_raise_like_slow_path(case):
    conf = _job()
    items = list(conf["edges"].items())
    (u, v), j = items[10]
    bad = {
        "dup": items + [((u, v), 2.0)],
        "dup_reversed": items + [((v, u), 2.0)],
        "neg": _mutate(conf["edges"], 5, ((-1, 3), 1.0)),
        "self": _mutate(conf["edges"], 5, ((4, 4), 1.0)),
        "np_int": _mutate(conf["edges"], 5, ((np.int64(4), 7), 1.0)),
        "str_coupling": _mutate(conf["edges"], 5, ((4, 7), "1.0")),
        "short": _mutate(conf["edges"], 5, ((4,), 1.0)),
    }[case]
    bad_conf = dict(conf, edges=bad)
    assert cfg._edges_fast(bad) is None
    with pytest.raises(cfg.ConfigSyntaxError) as slow:
        cfg.analyse_config(bad_conf)
    with pytest.raises(cfg.ConfigSyntaxError) as fast:
        cfg.analyse_config(bad_conf, edge_arrays=True)
    chain = lambda e: [str(x) for x in (e, e.__cause__, e.__cause__.__cause__ if e.__cause__ else None)]
    assert chain(fast.value) == chain(slow.value)


def test_bool_and_float_subclasses_accepted_like_slow_path():
    conf = _job()
    items = list(conf["edges"].items())
    items[3] = (items[3][0], True)
    items[4] = (items[4][0], np.float64(0.25))
    conf = dict(conf, edges=items)
    fast = cfg.analyse_config(conf, edge_arrays=True)[cfg.EDGES_KEY]
    slow = cfg.analyse_config(conf)[cfg.EDGES_KEY]
    assert np.array_equal(fast.ampl, np.array(list(slow.values())))


def test_duplicate_node_ids_in_list_form():
    conf = _job(form="list")
    conf["nodes"].append([3, 0.5])
    with pytest.raises(cfg.ConfigSyntaxError):
        cfg.analyse_config(conf, edge_arrays=True)


def test_build_context_unchanged_by_fast_path(monkeypatch):
    conf = _job(n=2000)
    a = build_context(conf)
    monkeypatch.setattr(cfg, "FAST_EDGES_MIN", 10 ** 9)
    b = build_context(conf)
    assert list(a.degree_to_layout) == list(b.degree_to_layout)
    for d, L in a.degree_to_layout.items():
        M = b.degree_to_layout[d]
        for f in ("node_ids", "input_msgs_position", "output_msgs_position", "lmbds_position", "node_ampls",
                  "edge_ampls"):
            assert np.array_equal(getattr(L, f), getattr(M, f))
    assert np.array_equal(a.node_ampl, b.node_ampl)
