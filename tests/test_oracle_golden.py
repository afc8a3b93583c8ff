"""Pin the CPU oracle against outputs recorded from the reference itself.

``tests/golden/*.npz`` were produced by ``tests/golden/make_golden.py``, which runs the
reference bqa numpy backend at FP64.  The oracle restatement must reproduce them to
round-off, which makes it a trustworthy checker for the GPU path.  Also: exactness of the
<Z Z> / density restatement on a tree (BP is exact on trees).
"""
import numpy as np
import pytest

from oracle import bqa_oracle as orc
from tests import golden_cases as gc

SMALL = gc.case_names(max_nodes=64)


@pytest.mark.parametrize("name", SMALL)
def test_oracle_reproduces_reference(name):
    conf = gc.config(name)
    want = gc.arrays(name)
    ctx = orc.make_context(conf)
    st = orc.initialize_state(ctx)
    dims, results = [], []
    for ins in ctx.instructions:
        if isinstance(ins, dict):
            orc.run_layer(ctx, ins["xtime"], ins["ztime"], st)
            dims.append(st.bond_dim)
        elif ins == "get_bloch_vectors":
            results.append(orc.bloch_vectors(orc.get_density_matrices(ctx, st)))
        elif ins == "measure":
            results.append(np.array(orc.measure(ctx, st)))
    assert dims == list(want["dims"])
    assert np.allclose(st.lmbds.real, want["lmbds"], atol=1e-9)
    for i, kind in enumerate(gc.manifest()[name]["results"]):
        got = results[i]
        ref = want[f"result{i}_{kind}"]
        if kind == "bloch_vectors":
            assert np.abs(got - ref).max() < 1e-9
        else:
            assert np.array_equal(got, ref)


@pytest.mark.slow
def test_oracle_reproduces_reference_c1():
    name = "c1_rr3_n1000_chi4"
    if name not in gc.case_names():
        pytest.skip("C1 fixture not generated")
    out = orc.run_qa(gc.config(name))
    ref = gc.arrays(name)["result0_bloch_vectors"]
    assert np.abs(np.array(out[0][1]) - ref).max() < 1e-8


def _tree_state(seed):
    conf = gc.config("tree9")
    ctx = orc.make_context(conf)
    st = orc.initialize_state(ctx)
    for ins in ctx.instructions[:6]:
        orc.run_layer(ctx, ins["xtime"], ins["ztime"], st)
    orc.run_bp(ctx, st)
    return ctx, st


def _contract_tree(ctx, st):
    """Dense state vector of the 9-node tree tensor network (exact contraction)."""
    n = ctx.nodes_number
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    bond_letter = {}
    nxt = [n]
    def letter(e):
        key = tuple(sorted(e))
        if key not in bond_letter:
            bond_letter[key] = letters[nxt[0]]
            nxt[0] += 1
        return bond_letter[key]
    ops, subs = [], []
    for v in range(n):
        d, pos = ctx.path_to_tensors[v]
        ops.append(st.degree_to_tensor[d][pos])
        subs.append(letters[v] + "".join(letter((v, u)) for u in ctx.graph[v]))
    psi = np.einsum(",".join(subs) + "->" + letters[:n], *ops)
    return psi / np.linalg.norm(psi)


def test_zz_and_density_restatement_exact_on_tree():
    ctx, st = _tree_state(0)
    psi = _contract_tree(ctx, st)
    n = ctx.nodes_number
    probs = np.abs(psi) ** 2
    zs = []
    for v in range(n):
        sign = np.ones([2] * n)
        idx = [slice(None)] * n
        idx[v] = 1
        sign[tuple(idx)] = -1
        zs.append(sign)
    z_exact = np.array([np.sum(probs * zs[v]) for v in range(n)])
    bloch = orc.bloch_vectors(orc.get_density_matrices(ctx, st))
    assert np.abs(bloch[:, 2] - z_exact).max() < 1e-8
    zz = orc.edge_zz(ctx, st)
    half = ctx.edges_number // 2
    keys = list(ctx.edge_to_ampl.keys())[:half]
    zz_exact = np.array([np.sum(probs * zs[a] * zs[b]) for a, b in keys])
    assert np.abs(zz - zz_exact).max() < 1e-8
    e = orc.energy(ctx, zz, bloch[:, 2])
    J = np.array([ctx.edge_to_ampl[k] for k in keys])
    h = np.array([ctx.node_to_ampl[v] for v in range(n)])
    assert abs(e - (J @ zz_exact + h @ z_exact)) < 1e-8
