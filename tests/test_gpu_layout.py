"""Device layout compiler (bqa_layout_degrees + bqa_layout_class) against the host compiler.

The host compiler is pinned bit-exact to the reference's known-answer test
(tests/test_config_layout.py); here the device compiler must give the same classes, class
order, node ids, slot maps and positions, bit for bit, including degree-0 nodes, mixed
degrees and large graphs, and turn bad edge lists into errors.
"""
import numpy as np
import pytest

from bqa_gb300 import instances, layout
from tests import golden_cases as gc
from tests.test_config_layout import KNOWN_CONFIG

pytestmark = pytest.mark.gpu


def _directed(und: np.ndarray) -> np.ndarray:
    und = np.asarray(und, dtype=np.int64).reshape(-1, 2)
    return np.concatenate([und, und[:, ::-1]], axis=0)


def _same(host, dev):
    hc, hdeg, hpos = host
    dc, ddeg, dpos = dev
    assert list(hc) == list(dc)                      # class order (first appearance)
    for d in hc:
        assert np.array_equal(hc[d][0], dc[d][0]), d
        assert hc[d][1].shape == dc[d][1].shape, d
        assert np.array_equal(hc[d][1], dc[d][1]), d
    assert np.array_equal(hdeg, ddeg)
    assert np.array_equal(hpos, dpos)


@pytest.mark.parametrize("n,d,seed", [(10, 3, 0), (1000, 3, 1), (20000, 4, 2), (200_000, 3, 3)])
def test_regular(n, d, seed):
    e = _directed(instances.random_regular_edges(n, d, seed))
    _same(layout.compile_layout(e, n), layout.compile_layout_device(e, n))


def test_mixed_degrees_and_isolated_nodes():
    rng = np.random.default_rng(5)
    degs = rng.choice([1, 2, 3, 5, 6], size=3000)
    degs[-1] += int(degs.sum() % 2)
    e = _directed(instances.configuration_model_edges(degs, 7))
    n = 3000 + 40                                    # 40 nodes without edges: the degree-0 class
    perm = rng.permutation(n)                        # scatter node ids so classes interleave
    e = perm[e]
    _same(layout.compile_layout(e, n), layout.compile_layout_device(e, n))


def test_grid_union():
    g = instances.periodic_grid_edges(30, 30)
    r = instances.random_regular_edges(500, 3, 9) + 900
    e = _directed(np.concatenate([g, r]))
    _same(layout.compile_layout(e, 1400), layout.compile_layout_device(e, 1400))


@pytest.mark.parametrize("name", ["known"] + gc.case_names())
def test_contexts_identical(name, monkeypatch):
    conf = KNOWN_CONFIG if name == "known" else gc.config(name)
    host = layout.build_context(conf)
    monkeypatch.setattr(layout, "DEVICE_LAYOUT_MIN_EDGES", 0)
    dev = layout.build_context(conf, layout_device="cuda")
    assert list(host.degree_to_layout) == list(dev.degree_to_layout)
    for d, L in host.degree_to_layout.items():
        M = dev.degree_to_layout[d]
        for f in ("node_ids", "input_msgs_position", "output_msgs_position", "lmbds_position", "node_ampls",
                  "edge_ampls"):
            assert np.array_equal(getattr(L, f), getattr(M, f)), (d, f)
    assert np.array_equal(host.node_degree, dev.node_degree)
    assert np.array_equal(host.node_position, dev.node_position)


def test_bad_edges_are_errors():
    e = _directed(np.array([[0, 1], [1, 2], [2, 3]]))
    bad = e.copy()
    bad[1] = [7, 1]                                  # endpoint outside [0, n)
    with pytest.raises(ValueError):
        layout.compile_layout_device(bad, 4)
    bad = e.copy()
    bad[4] = [1, 0]                                  # slot 1 + E/2 is not the reversal of slot 1
    with pytest.raises(ValueError):
        layout.compile_layout_device(bad, 4)
    star = _directed(np.array([[0, k] for k in range(1, 10)]))
    with pytest.raises(ValueError):
        layout.compile_layout_device(star, 10, max_degree=4)
    _same(layout.compile_layout(star, 10), layout.compile_layout_device(star, 10, max_degree=9))
