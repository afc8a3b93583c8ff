"""The FP32-accurate tensor-core (tcgen05) half-node message kernels of degree 3 at bond dim 16.

BQA_VARIANT_TENSOR runs the bond products T x_k M_k and the closing contractions on the tensor
cores in 2xFP16 (BQA_GB300_TC_KIND at load selects 2xFP16 products with CUDA-core closing
contractions, or 3xTF32 products).  Checked through the C ABI (bqa_bp_sweep_plan with
BQA_VARIANT_TENSOR, and the default two-stage entry points that launch it):
  * one BP sweep equals one oracle sweep to the complex64 kernel tolerance (2e-5 relative);
  * it agrees with the CUDA-core half-node kernel (BQA_VARIANT_TILED) to 2e-6 relative on a
    few hundred nodes with dense random Hermitian messages;
  * diagonal incoming messages (the first sweep after a truncation) match the oracle;
  * the extended messages of the two-stage pass match the oracle;
  * the per-half-node FP16 operand scaling leaves normalised messages unchanged for tensors
    and messages far from unit scale;
  * no CTA ever hits the bounded wait for its MMAs (bqa_tc_faults stays 0);
  * other shapes are refused with BQA_ERR_UNSUPPORTED.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib, instances  # noqa: E402
from bqa_gb300.engine import Annealer, _ptr  # noqa: E402
from bqa_gb300.layout import build_context  # noqa: E402
from oracle import bqa_oracle as orc  # noqa: E402
from tests.test_gpu_kernels import RTOL, random_state, rel_err  # noqa: E402


def oracle_sweep(octx, msgs, tens):
    want = np.empty_like(msgs)
    for d, t in tens.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [msgs[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    return want


def plan_sweep(job, variant):
    arr = (ctypes.c_int32 * len(job.classes))(*([variant] * len(job.classes)))
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_plan", job._class_array(), len(job.classes), job.chis, job.dtype, arr,
                 _ptr(job.msgs[0]), _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), None, job.stream)
    return job.msgs[1][: job.E * job.chis * job.chis].cpu().numpy().reshape(job.E, job.chis, job.chis)


def dense_state(n, seed, chi=16):
    """A random 3-regular instance with random normalised tensors and random PSD messages."""
    edges = instances.random_regular_edges(n, 3, seed)
    rng = np.random.default_rng(seed)
    conf = instances.qubo_config(edges, rng.normal(size=len(edges)), rng.normal(size=n), max_bond_dim=chi,
                                 schedule=instances.anneal_schedule(1.0, 1))
    ctx = build_context(conf)
    tens = {}
    for d, L in ctx.degree_to_layout.items():
        shape = (L.batch_size, 2) + (chi,) * d
        t = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        t /= np.linalg.norm(t.reshape(shape[0], -1), axis=1).reshape((-1,) + (1,) * (t.ndim - 1))
        tens[d] = t.astype(np.complex64).astype(np.complex128)
    E = ctx.edges_number
    a = rng.normal(size=(E, chi, chi)) + 1j * rng.normal(size=(E, chi, chi))
    m = a @ np.conj(np.swapaxes(a, 1, 2)) + 0.1 * np.eye(chi)
    m /= np.trace(m, axis1=1, axis2=2)[:, None, None]
    m = m.astype(np.complex64).astype(np.complex128)
    job = Annealer(ctx, precision="single", pad_bonds=False)
    job.set_state(tens, m)
    return ctx, tens, m, job


def test_tensor_core_sweep_matches_oracle():
    octx, st, job = random_state("rr3_n16_chi4", 16, seed=4)
    want = oracle_sweep(octx, st.msgs, st.degree_to_tensor)
    got = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
    err = rel_err(got, want)
    print(f"tensor-core sweep vs oracle: {err:.2e}")
    assert err < RTOL
    assert job.lib.tc_faults(job.stream) == 0


@pytest.mark.parametrize("n,seed", [(64, 1), (512, 2)])
def test_tensor_core_sweep_matches_cuda_core_kernel(n, seed):
    ctx, tens, m, job = dense_state(n, seed)
    tc = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
    cc = plan_sweep(job, _lib.BQA_VARIANT_TILED)
    err = rel_err(tc, cc)
    print(f"n={n}: tensor-core vs CUDA-core sweep {err:.2e}")
    assert err < 2e-6
    if n <= 64:
        want = oracle_sweep(ctx, m, tens)
        assert rel_err(tc, want) < RTOL
    assert job.lib.tc_faults(job.stream) == 0


_DEFAULT_SCRIPT = """
import sys, ctypes, numpy as np
from tests.test_gpu_tensor_core import dense_state, plan_sweep
from bqa_gb300 import _lib
from bqa_gb300.engine import _ptr
ctx, tens, m, job = dense_state(128, 3)
tc = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
job.dist_parts.zero_()
job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), 16, job.dtype, _ptr(job.msgs[0]),
             _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), None, job.stream)
got = job.msgs[1][: job.E * 256].cpu().numpy().reshape(job.E, 16, 16)
sys.exit(0 if np.array_equal(got, tc) else 3)
"""


def test_tensor_core_kernel_as_the_default_two_stage_sweep():
    """With BQA_GB300_TC=1 at load (the default), bqa_bp_sweep_split at (3, 16) gives the TENSOR
    variant's bits."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, BQA_GB300_TC="1", PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", _DEFAULT_SCRIPT], cwd=root, env=env, timeout=600)
    assert r.returncode == 0


def test_tensor_core_kernel_with_diagonal_messages():
    octx, st, job = random_state("rr3_n16_chi4", 16, seed=11)
    rng = np.random.default_rng(5)
    lam = rng.uniform(0.1, 1.0, size=(octx.edges_number, 16))
    m = np.zeros((octx.edges_number, 16, 16), dtype=np.complex128)
    m[:, np.arange(16), np.arange(16)] = lam / lam.sum(axis=1, keepdims=True)
    m = m.astype(np.complex64).astype(np.complex128)
    job.set_state(st.degree_to_tensor, m)
    want = oracle_sweep(octx, m, st.degree_to_tensor)
    got = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
    assert rel_err(got, want) < RTOL
    # one off-diagonal entry of 1e-30 per message: the dense tensor-core products, same values
    m2 = m.copy()
    m2[:, 0, 15] = 1e-30
    job.set_state(st.degree_to_tensor, m2)
    dense = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
    assert rel_err(dense, got) < 1e-6


def test_tensor_core_extended_messages_match_oracle():
    octx, st, job = random_state("rr3_n16_chi4", 16, seed=7)
    zt = 0.37
    job.lib.call("bqa_ext_msgs_split", job._class_array(), len(job.classes), 16, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.lu), job.E, _ptr(job.edge_j), zt, _ptr(job.ext), job.stream)
    want = orc.get_extended_msgs(octx, zt, st)
    got = job.ext[: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < RTOL


_KIND_SCRIPT = """
import sys, numpy as np
from tests.test_gpu_tensor_core import dense_state, plan_sweep
from tests.test_gpu_kernels import rel_err
from bqa_gb300 import _lib
from tests.test_gpu_tensor_core import oracle_sweep
ctx, tens, m, job = dense_state(128, 3)
tc = plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
cc = plan_sweep(job, _lib.BQA_VARIANT_TILED)
err, err_o = rel_err(tc, cc), rel_err(tc, oracle_sweep(ctx, m, tens))
print(f"tensor-core kernel {sys.argv[1]!r}: vs CUDA-core sweep {err:.2e}, vs oracle {err_o:.2e}")
sys.exit(0 if err < 2e-6 and err_o < 2e-6 and job.lib.tc_faults(job.stream) == 0 else 3)
"""


@pytest.mark.parametrize("kind", ["products", "tf32"])
def test_other_tensor_core_kernels_match_cuda_core_kernel(kind):
    """BQA_GB300_TC_KIND at load selects 2xFP16 products with CUDA-core closing contractions
    ("products") or 3xTF32 products ("tf32") for BQA_VARIANT_TENSOR; both are FP32-accurate."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, BQA_GB300_TC_KIND=kind, PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", _KIND_SCRIPT, kind], cwd=root, env=env, timeout=600)
    assert r.returncode == 0


def _normalised(m):
    return m / np.trace(m, axis1=1, axis2=2)[:, None, None]


def test_tensor_core_sweep_scaling_of_operands():
    """The FP16 operands are scaled per half-node: tensors scaled by 2^-40 (beyond the scale
    exponent's clamp) and messages by 2^20 give the same normalised messages."""
    ctx, tens, m, job = dense_state(64, 6)
    base = _normalised(plan_sweep(job, _lib.BQA_VARIANT_TENSOR))
    job.set_state({d: t * 2.0 ** -40 for d, t in tens.items()}, m * 2.0 ** 20)
    scaled = _normalised(plan_sweep(job, _lib.BQA_VARIANT_TENSOR))
    err = rel_err(scaled, base)
    print(f"scaled operands: {err:.2e}")
    assert err < 2e-6
    assert job.lib.tc_faults(job.stream) == 0


def test_tensor_variant_refuses_other_shapes():
    octx, st, job = random_state("rr3_n24_chi8", 8, seed=1)
    with pytest.raises(_lib.BqaError) as e:
        plan_sweep(job, _lib.BQA_VARIANT_TENSOR)
    assert e.value.status == _lib.BQA_ERR_UNSUPPORTED


# ---- BF16 tensor-core kernel and the mixed-precision kernel --------------------------------

BF16_RTOL = 2e-2   # BF16 operands (8-bit significands), FP32 accumulation


def plan_sweep_ls(job, variant, loop_state):
    """One two-stage sweep through bqa_bp_sweep_plan with a device loop state (reads buffer 0)."""
    arr = (ctypes.c_int32 * len(job.classes))(*([variant] * len(job.classes)))
    ls = torch.as_tensor(np.asarray(loop_state, dtype=np.int32), device=job.msgs[0].device)
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_plan", job._class_array(), len(job.classes), job.chis, job.dtype, arr,
                 _ptr(job.msgs[0]), _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), _ptr(ls),
                 job.stream)
    return job.msgs[1][: job.E * job.chis * job.chis].cpu().numpy().reshape(job.E, job.chis, job.chis)


def loop_state(sweeps, dist):
    ls = np.zeros(8, dtype=np.int32)
    ls[1] = sweeps
    ls[5] = np.array([dist], dtype=np.float32).view(np.int32)[0]
    return ls


def test_bf16_sweep_matches_oracle_to_bf16_precision():
    octx, st, job = random_state("rr3_n16_chi4", 16, seed=4)
    want = oracle_sweep(octx, st.msgs, st.degree_to_tensor)
    got = plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16)
    err = rel_err(got, want)
    print(f"bf16 tensor-core sweep vs oracle: {err:.2e}")
    assert err < BF16_RTOL
    assert job.lib.tc_faults(job.stream) == 0


@pytest.mark.parametrize("n,seed", [(64, 1), (512, 2)])
def test_bf16_sweep_matches_fp32_kernel(n, seed):
    ctx, tens, m, job = dense_state(n, seed)
    lo = plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16)
    hi = plan_sweep(job, _lib.BQA_VARIANT_TILED)
    err = rel_err(lo, hi)
    # messages of different slots come out of independent blocks: every slot within the bound
    per_slot = np.abs(lo - hi).max(axis=(1, 2)) / np.abs(hi).max(axis=(1, 2))
    print(f"n={n}: bf16 vs fp32 sweep {err:.2e} (worst slot {per_slot.max():.2e})")
    assert err < BF16_RTOL and per_slot.max() < 5 * BF16_RTOL
    # unit trace (the combine kernel's normalisation); Hermitian to BF16 rounding: the tensor
    # cores form every entry of a block, not its upper triangle and a mirror (measured 6e-5)
    assert np.abs(np.trace(lo, axis1=1, axis2=2) - 1).max() < 1e-5
    assert np.abs(lo - np.conj(np.swapaxes(lo, 1, 2))).max() < 5e-4
    assert job.lib.tc_faults(job.stream) == 0


def test_bf16_kernel_with_diagonal_messages_is_exact():
    """Diagonal incoming messages: the bond-scaling path in FP32, as in the FP32 kernels."""
    octx, st, job = random_state("rr3_n16_chi4", 16, seed=11)
    rng = np.random.default_rng(5)
    lam = rng.uniform(0.1, 1.0, size=(octx.edges_number, 16))
    m = np.zeros((octx.edges_number, 16, 16), dtype=np.complex128)
    m[:, np.arange(16), np.arange(16)] = lam / lam.sum(axis=1, keepdims=True)
    m = m.astype(np.complex64).astype(np.complex128)
    job.set_state(st.degree_to_tensor, m)
    want = oracle_sweep(octx, m, st.degree_to_tensor)
    assert rel_err(plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16), want) < RTOL
    assert np.array_equal(plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16), plan_sweep(job, _lib.BQA_VARIANT_TILED))


def test_mixed_kernel_follows_the_loop_state():
    """BF16 path after the first sweep while the last distance is above the switch (2^-5), the
    default FP32-accurate kernel otherwise (bit-identical to it: the 2xFP16 tensor-core kernel,
    or the CUDA-core kernel with BQA_GB300_TC=0), FP32 without a loop state."""
    import os
    ctx, tens, m, job = dense_state(128, 7)
    tc_default = os.environ.get("BQA_GB300_TC", "1") != "0"
    fp32 = plan_sweep(job, _lib.BQA_VARIANT_TENSOR if tc_default else _lib.BQA_VARIANT_TILED)
    bf16 = plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16)
    assert not np.array_equal(fp32, bf16)
    assert np.array_equal(plan_sweep(job, _lib.BQA_VARIANT_MIXED), fp32)                     # no loop state
    assert np.array_equal(plan_sweep_ls(job, _lib.BQA_VARIANT_MIXED, loop_state(3, 0.5)), bf16)
    assert np.array_equal(plan_sweep_ls(job, _lib.BQA_VARIANT_MIXED, loop_state(3, 1e-3)), fp32)
    assert np.array_equal(plan_sweep_ls(job, _lib.BQA_VARIANT_MIXED, loop_state(0, 0.5)), fp32)  # first sweep
    assert job.lib.tc_faults(job.stream) == 0


def test_bf16_kernel_mixes_diagonal_and_dense_nodes():
    """Nodes whose incoming messages are all diagonal take the FP32 bond-scaling path
    (bit-identical to the CUDA-core kernel), the others the BF16 tensor-core path, within one
    launch."""
    ctx, tens, m, job = dense_state(2048, 9)
    L = ctx.degree_to_layout[3]
    diag_nodes = np.arange(L.batch_size) % 3 == 0
    m = m.copy()
    for k in range(3):
        slots = L.input_msgs_position[k][diag_nodes]
        d = np.real(np.diagonal(m[slots], axis1=1, axis2=2))
        m[slots] = 0
        m[slots[:, None], np.arange(16), np.arange(16)] = d / d.sum(axis=1, keepdims=True)
    m = m.astype(np.complex64).astype(np.complex128)
    job.set_state(tens, m)
    all_diag = np.ones(L.batch_size, dtype=bool)
    for k in range(3):
        sl = L.input_msgs_position[k]
        off = np.abs(m[sl] - np.einsum("eii->ei", m[sl])[:, :, None] * np.eye(16)).max(axis=(1, 2))
        all_diag &= off == 0
    assert all_diag.sum() > 0 and (~all_diag).sum() > 0
    lo = plan_sweep(job, _lib.BQA_VARIANT_TENSOR_BF16)
    hi = plan_sweep(job, _lib.BQA_VARIANT_TILED)
    exact = L.output_msgs_position[:, all_diag].ravel()
    approx = L.output_msgs_position[:, ~all_diag].ravel()
    # a slot's message is (P_0 + P_1) of one node: exact where that node took the FP32 path
    assert np.array_equal(lo[exact], hi[exact])
    assert rel_err(lo[approx], hi[approx]) < BF16_RTOL
    assert job.lib.tc_faults(job.stream) == 0
