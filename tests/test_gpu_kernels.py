"""Kernel-level parity of the CUDA path against the FP64 oracle, on identical seeded inputs.

Each test loads one random state (complex tensors at a fixed bond dim, random PSD
trace-normalised messages) into the device engine, runs one C-ABI entry point and compares
with the oracle function the kernel restates.  Tolerances are for complex64 arithmetic:
deterministic outputs (messages, extended messages, updated tensors, densities) to 2e-5
relative to their largest entry; gauge-dependent outputs only through gauge-invariant
combinations.
"""
import numpy as np
import pytest

from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib  # noqa: E402
from bqa_gb300.engine import Annealer, _ptr  # noqa: E402
from bqa_gb300.layout import build_context  # noqa: E402
from oracle import bqa_oracle as orc  # noqa: E402

# (case, bond dim): register-tiled kernels for (d, chi) in {2,3,4} x {4,8,12,16} (chi % 4 == 0
# where built), the generic kernel elsewhere (mixed degrees up to 7, odd chi, degree 1)
CASES = [("rr3_n16_chi4", 4), ("rr3_n24_chi8", 8), ("mixed_n18_chi3", 3), ("rr4_n20_chi4", 4),
         ("rr3_n16_chi4", 16), ("grid3x4_chi4_damped", 5), ("tree9", 2), ("grid3x4_chi4_damped", 8),
         ("rr3_n24_chi8", 12), ("grid3x4_chi4_damped", 4),
         # degree-7 node tensors beyond shared memory: the global-memory kernels
         ("mixed_n18_chi3", 4),
         # bond dim 32: global-memory kernels and the 64-column Jacobi
         ("rr3_n16_chi4", 32)]
RTOL = 2e-5


def random_state(name, chi, seed=0, precision="single"):
    conf = gc.config(name)
    conf["max_bond_dim"] = chi
    octx = orc.make_context(conf)
    rng = np.random.default_rng(seed)
    tens = {}
    for d, L in octx.degree_to_layout.items():
        shape = (L.node_ids.shape[0], 2) + (chi,) * d
        t = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        t /= np.linalg.norm(t.reshape(shape[0], -1), axis=1).reshape((-1,) + (1,) * (t.ndim - 1))
        tens[d] = t
    a = rng.normal(size=(octx.edges_number, chi, chi)) + 1j * rng.normal(size=(octx.edges_number, chi, chi))
    m = a @ np.conj(np.swapaxes(a, 1, 2)) + 0.1 * np.eye(chi)
    m /= np.trace(m, axis1=1, axis2=2)[:, None, None]
    lam = np.sort(rng.uniform(0.05, 1.0, size=(octx.edges_number // 2, chi)), axis=1)[:, ::-1]
    lam /= np.linalg.norm(lam, axis=1, keepdims=True)
    # round to complex64 so both sides see the same inputs
    tens = {d: t.astype(np.complex64).astype(np.complex128) for d, t in tens.items()}
    m = m.astype(np.complex64).astype(np.complex128)
    st = orc.OracleState(np.random.default_rng(0), tens, m, lam.astype(np.complex128))
    job = Annealer(build_context(conf), precision=precision, pad_bonds=False)
    job.set_state(tens, m, lam)
    return octx, st, job


def rel_err(got, want):
    return float(np.abs(got - want).max() / max(np.abs(want).max(), 1e-30))


@pytest.mark.parametrize("name,chi", CASES)
def test_bp_sweep_matches_oracle(name, chi):
    octx, st, job = random_state(name, chi)
    want = np.empty_like(st.msgs)
    for d, t in st.degree_to_tensor.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [st.msgs[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.msgs[1]), _ptr(job.dist_parts), None, job.stream)
    got = job.msgs[1][: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < RTOL
    num, den = job.dist_parts.view(torch.int32)[:2].view(torch.float32).cpu().numpy()
    d_want = orc.get_dist(want, st.msgs)
    assert abs(np.sqrt(num) / np.sqrt(den) - d_want) < 1e-5 * max(1.0, d_want)


@pytest.mark.parametrize("name,chi", CASES)
@pytest.mark.parametrize("precision", ["single", "double"])
def test_split_bp_sweep_matches_oracle(name, chi, precision):
    """Two-stage sweep (open-bond blocks through scratch, then messages) = one oracle sweep."""
    if precision == "double" and chi > 5:
        pytest.skip("complex128 node kernels hold a smaller bond dim (6 at degree 4)")
    octx, st, job = random_state(name, chi, seed=9, precision=precision)
    want = np.empty_like(st.msgs)
    for d, t in st.degree_to_tensor.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [st.msgs[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.msgs[1]), _ptr(job.lu), octx.edges_number, _ptr(job.dist_parts), None, job.stream)
    got = job.msgs[1][: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < (RTOL if precision == "single" else 1e-12)
    parts = job.dist_parts.cpu()
    if precision == "single":
        num, den = parts.view(torch.int32)[:2].view(torch.float32).numpy()
    else:
        num, den = parts.view(torch.float64).numpy()
    d_want = orc.get_dist(want, st.msgs)
    assert abs(np.sqrt(num) / np.sqrt(den) - d_want) < 1e-5 * max(1.0, d_want)


@pytest.mark.parametrize("name,chi", [("rr3_n16_chi4", 16), ("rr3_n24_chi8", 8), ("rr3_n24_chi8", 12),
                                      ("rr3_n16_chi4", 4)])
def test_split_sweep_with_diagonal_messages_matches_oracle(name, chi):
    """Diagonal incoming messages (the first sweep after a truncation, diag(lambda)/tr): the
    degree-3 half-node kernels detect them and apply them as bond scalings; one oracle sweep
    to the complex64 tolerance, and the dense products' values (to 1e-6) when one off-diagonal
    entry of 1e-30 per message makes the kernels take the dense path."""
    octx, st, job = random_state(name, chi, seed=11)
    rng = np.random.default_rng(5)
    lam = rng.uniform(0.1, 1.0, size=(octx.edges_number, chi))
    m = np.zeros((octx.edges_number, chi, chi), dtype=np.complex128)
    m[:, np.arange(chi), np.arange(chi)] = lam / lam.sum(axis=1, keepdims=True)
    m = m.astype(np.complex64).astype(np.complex128)
    st.msgs = m
    job.set_state(st.degree_to_tensor, m)
    want = np.empty_like(m)
    for d, t in st.degree_to_tensor.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [m[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.msgs[1]), _ptr(job.lu), octx.edges_number, _ptr(job.dist_parts), None, job.stream)
    got = job.msgs[1][: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < RTOL
    # one off-diagonal entry of 1e-30 per message sends the kernels down the dense products
    m2 = m.copy()
    m2[:, 0, chi - 1] = 1e-30
    job.set_state(st.degree_to_tensor, m2)
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.msgs[1]), _ptr(job.lu), octx.edges_number, _ptr(job.dist_parts), None, job.stream)
    dense = job.msgs[1][: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, dense) < 1e-6
@pytest.mark.parametrize("name,chi", CASES)
def test_ext_msgs_match_oracle(name, chi):
    octx, st, job = random_state(name, chi, seed=1)
    ztime = 0.37
    want = orc.get_extended_msgs(octx, ztime, st)
    job.lib.call("bqa_ext_msgs", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.ext), ztime, job.stream)
    got = job.ext[: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < RTOL


@pytest.mark.parametrize("name,chi", CASES)
@pytest.mark.parametrize("precision", ["single", "double"])
def test_ext_msgs_split_matches_oracle_and_one_pass(name, chi, precision):
    """Two-stage extended messages (half-node blocks + per-slot combine) against the oracle
    and against the one-pass kernel (same epilogue arithmetic; the blocks' K-split can
    differ between the half-node and whole-node launch shapes, so agreement is to rounding)."""
    if precision == "double" and chi > 5:
        pytest.skip("complex128 node kernels hold a smaller bond dim (6 at degree 4)")
    octx, st, job = random_state(name, chi, seed=1, precision=precision)
    ztime = 0.37
    want = orc.get_extended_msgs(octx, ztime, st)
    job.lib.call("bqa_ext_msgs_split", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.lu), job.E, _ptr(job.edge_j), ztime, _ptr(job.ext), job.stream)
    got = job.ext[: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < (RTOL if precision == "single" else 1e-12)
    job.lib.call("bqa_ext_msgs", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.ul), ztime, job.stream)
    one = job.ul[: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, one) < (2e-6 if precision == "single" else 1e-14)


@pytest.mark.parametrize("name,chi", CASES)
def test_canonicalisers_match_oracle(name, chi):
    octx, st, job = random_state(name, chi, seed=2)
    ext = orc.get_extended_msgs(octx, 0.21, st).astype(np.complex64).astype(np.complex128)
    eps = octx.pinv_eps
    lam_w, can_w = orc.get_canonicalizers(ext, eps)
    E, n = ext.shape[0], ext.shape[1]
    job.ext[: ext.size].copy_(torch.from_numpy(ext.astype(np.complex64).reshape(-1)))
    job.status.zero_()
    job.colmax.zero_()
    job.lib.call("bqa_env_factor", _ptr(job.ext), E, n, job.dtype, eps, _ptr(job.lu), _ptr(job.ul), _ptr(job.status),
                 job.stream)
    job.lib.call("bqa_bond_canon", _ptr(job.lu), _ptr(job.ul), E, n, job.dtype, eps, _ptr(job.ext), _ptr(job.lmbds),
                 _ptr(job.colmax), _ptr(job.status), job.stream)
    assert int(job.status.item()) == 0
    lam = job.lmbds[: E // 2 * n].cpu().numpy().reshape(E // 2, n)
    can = job.ext[: E * n * n].cpu().numpy().reshape(E, n, n)
    big = lam_w.real > 1e-3
    assert np.abs(lam - lam_w.real)[big].max() < 2e-5
    colmax = job.colmax[:n].view(torch.float32).cpu().numpy()
    assert np.allclose(colmax, lam.max(axis=0))
    # gauge-invariant bond operator  can[p+h] diag(lam) can[p]^T  (= P_fwd P_bwd^T, projectors)
    h = E // 2
    keep = (lam_w.real > 1e-3).astype(float)
    g_w = np.einsum("pic,pc,pjc->pij", can_w[h:], lam_w.real * keep, can_w[:h])
    g = np.einsum("pic,pc,pjc->pij", can[h:], lam * keep, can[:h])
    assert rel_err(g, g_w) < 5e-4


@pytest.mark.parametrize("name,chi,dim", [("rr3_n16_chi4", 2, 4), ("rr3_n24_chi8", 8, 8), ("grid3x4_chi4_damped", 3, 5),
                                          ("rr4_n20_chi4", 4, 3), ("rr3_n16_chi4", 16, 16)])
def test_apply_update_matches_oracle(name, chi, dim):
    octx, st, job = random_state(name, max(chi, dim), seed=3)
    # re-draw a state at bond chi, and canonicalisers with n = 2 chi, dim columns
    rng = np.random.default_rng(4)
    tens = {}
    for d, L in octx.degree_to_layout.items():
        shape = (L.node_ids.shape[0], 2) + (chi,) * d
        tens[d] = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64).astype(np.complex128)
    E, n = octx.edges_number, 2 * chi
    can = (rng.normal(size=(E, n, n)) + 1j * rng.normal(size=(E, n, n))).astype(np.complex64).astype(np.complex128)
    lam = np.sort(rng.uniform(0.05, 1.0, size=(E // 2, n)), axis=1)[:, ::-1].astype(np.float32)
    ztime, xtime = 0.13, 0.41
    ost = orc.OracleState(np.random.default_rng(0), {d: t.copy() for d, t in tens.items()},
                          np.zeros((E, dim, dim), complex), lam[:, :dim].astype(np.complex128))
    for d, L in octx.degree_to_layout.items():
        aligned = [can[p][:, :, :dim] for p in L.input_msgs_position]
        ost.degree_to_tensor[d] = orc.apply_canonicalizers_with_extensions(
            ost.degree_to_tensor[d], aligned, [a * ztime for a in L.edge_ampls])
    orc.apply_z_layer(octx, ztime, ost)
    orc.apply_x_layer(xtime, ost)
    orc.set_to_symmetric_gauge(octx, ost)
    job.set_state(tens, np.zeros((E, chi, chi), np.complex64))
    job.ext[: can.size].copy_(torch.from_numpy(can.astype(np.complex64).reshape(-1)))
    job.lmbds[: lam.size].copy_(torch.from_numpy(lam.reshape(-1)))
    job.lib.call("bqa_apply_update", job._class_array(out=True), len(job.classes), chi, dim, job.dtype,
                 _ptr(job.ext), _ptr(job.lmbds), n, ztime, xtime, job.stream)
    job.tcur = 1
    job.chi = job.chis = dim
    for c in job.classes:
        shape = (c.count, 2) + (dim,) * c.degree
        got = c.tensors[1][: int(np.prod(shape))].cpu().numpy().reshape(shape)
        assert rel_err(got, ost.degree_to_tensor[c.degree]) < RTOL
    job.lib.call("bqa_msgs_from_lmbds", _ptr(job.lmbds), n, E, dim, job.dtype, _ptr(job.msgs[0]), job.stream)
    got_m = job.msgs[0][: E * dim * dim].cpu().numpy().reshape(E, dim, dim)
    assert rel_err(got_m, ost.msgs) < 1e-6


@pytest.mark.parametrize("name,chi", CASES)
def test_densities_and_zz_match_oracle(name, chi):
    octx, st, job = random_state(name, chi, seed=5)
    rho_w = orc.get_density_matrices(octx, st)
    rho = job.density_matrices()
    assert np.abs(rho - rho_w).max() < 2e-5
    zz_w = orc.edge_zz(octx, st)
    assert np.abs(job.edge_zz() - zz_w).max() < 2e-5


@pytest.mark.parametrize("name,chi", [("rr3_n16_chi4", 4), ("mixed_n18_chi3", 3), ("grid3x4_chi4_damped", 4)])
def test_bp_loop_matches_oracle(name, chi):
    octx, st, job = random_state(name, chi, seed=6)
    octx.bp_eps = 1e-6
    job.ctx.bp_eps = 1e-6
    orc.run_bp(octx, st)
    job.run_bp()
    _, msgs, _ = job.get_state()
    assert np.abs(msgs - st.msgs).max() < 2e-5


@pytest.mark.parametrize("name,chi", [("rr3_n16_chi4", 4), ("mixed_n18_chi3", 3), ("tree9", 2),
                                      ("mixed_n18_chi3", 4), ("rr3_n16_chi4", 20)])
def test_double_precision_kernels_match_oracle_to_roundoff(name, chi):
    """The complex128 build of the same kernels agrees with the FP64 oracle to ~1e-12."""
    octx, st, job = random_state(name, chi, seed=7, precision="double")
    want = np.empty_like(st.msgs)
    for d, t in st.degree_to_tensor.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [st.msgs[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.msgs[1]), _ptr(job.dist_parts), None, job.stream)
    got = job.msgs[1][: want.size].cpu().numpy().reshape(want.shape)
    assert rel_err(got, want) < 1e-12
    ext_w = orc.get_extended_msgs(octx, 0.3, st)
    job.lib.call("bqa_ext_msgs", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                 _ptr(job.ext), 0.3, job.stream)
    assert rel_err(job.ext[: ext_w.size].cpu().numpy().reshape(ext_w.shape), ext_w) < 1e-12
    assert np.abs(job.density_matrices() - orc.get_density_matrices(octx, st)).max() < 1e-12


@pytest.mark.parametrize("name,chi,maxd", [("rr3_n16_chi4", 6, 8), ("rr4_n20_chi4", 7, 8), ("grid3x4_chi4_damped", 5, 7),
                                           ("rr3_n24_chi8", 13, 16)])
def test_zero_padded_bond_storage_is_exact(name, chi, maxd):
    """A bond dim stored zero-padded to a multiple of 4 (tiled kernels) gives the same step as
    the unpadded generic path: same new bond dim, marginals and bond spectra within 1e-5."""
    conf = gc.config(name)
    conf["max_bond_dim"] = maxd
    octx, st, _ = random_state(name, chi, seed=8)
    runs = []
    for pad in (False, True):
        job = Annealer(build_context(conf), pad_bonds=pad)
        job.set_state(st.degree_to_tensor, st.msgs, st.lmbds)
        assert job.chis == (chi if not pad else chi + 4 - chi % 4)
        info = job.run_layer(0.07, 0.11)
        _, _, lam = job.get_state()
        runs.append((info["bond_dim"], job.bloch_vectors(), lam, job.edge_zz()))
    assert runs[0][0] == runs[1][0]
    assert np.abs(runs[0][1] - runs[1][1]).max() < 1e-5
    assert np.abs(runs[0][2] - runs[1][2]).max() < 1e-5
    assert np.abs(runs[0][3] - runs[1][3]).max() < 1e-5


_SWEEP_SCRIPT = """
import sys, numpy as np
from tests.test_gpu_kernels import random_state
from bqa_gb300.engine import _ptr
octx, st, job = random_state("rr3_n16_chi4", 16, seed=11)
job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), 16, job.dtype, _ptr(job.msgs[0]),
             _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), None, job.stream)
msgs = job.msgs[1][: job.E * 256].cpu().numpy()
job.lib.call("bqa_ext_msgs_split", job._class_array(), len(job.classes), 16, job.dtype, _ptr(job.msgs[0]),
             _ptr(job.lu), job.E, _ptr(job.edge_j), 0.37, _ptr(job.ext), job.stream)
ext = job.ext[: job.E * 1024].cpu().numpy()
import torch
rng = np.random.default_rng(5)
n, E = 32, job.E
can = (rng.normal(size=(E, n, n)) + 1j * rng.normal(size=(E, n, n))).astype(np.complex64)
lam = np.ascontiguousarray(np.sort(rng.uniform(0.05, 1.0, size=(E // 2, n)), axis=1)[:, ::-1].astype(np.float32))
job.ext[: can.size].copy_(torch.from_numpy(can.reshape(-1)))
job.lmbds[: lam.size].copy_(torch.from_numpy(lam.reshape(-1)))
job.lib.call("bqa_apply_update", job._class_array(out=True), len(job.classes), 16, 16, job.dtype, _ptr(job.ext),
             _ptr(job.lmbds), n, 0.13, 0.41, job.stream)
upd = job.classes[0].tensors[1][: job.classes[0].count * 2 * 4096].cpu().numpy()
np.savez(sys.argv[1], msgs=msgs, ext=ext, upd=upd)
"""


def test_specialised_half_kernel_bit_identical_to_generic(tmp_path):
    """The (3, 16) CUDA-core half-node kernel and tensor update with closed-form addresses give
    the generic kernels' bits (with the tensor-core kernel switched off)."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    out = {}
    for flag in ("1", "0"):
        env = dict(os.environ, BQA_GB300_SPECIALIZED=flag, BQA_GB300_TC="0", PYTHONPATH=str(root))
        f = tmp_path / f"spec{flag}.npz"
        subprocess.run([sys.executable, "-c", _SWEEP_SCRIPT, str(f)], cwd=root, env=env, check=True, timeout=600)
        out[flag] = np.load(f)
    assert np.array_equal(out["1"]["msgs"], out["0"]["msgs"])
    assert np.array_equal(out["1"]["ext"], out["0"]["ext"])
    assert np.array_equal(out["1"]["upd"], out["0"]["upd"])
    assert np.abs(out["1"]["msgs"]).max() > 0 and np.abs(out["1"]["upd"]).max() > 0


def test_fp32_fma_probe_runs():
    """The FP32 throughput probe (probe library) launches, writes every output and gives a
    plausible rate."""
    import bench
    probes = _lib.load_probes()
    out = torch.full((152 * 256,), float("nan"), device="cuda")
    assert probes.bqa_fp32_fma_probe(152, 10, _ptr(out), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    tf = bench.fp32_peak_tflops(torch.device("cuda"))
    assert 5.0 < tf < 500.0


def test_mma_probe_runs():
    """The warp-level MMA probe launches both kinds, writes every output, gives plausible rates."""
    import bench
    probes = _lib.load_probes()
    out = torch.full((152 * 256,), float("nan"), device="cuda")
    for kind in (0, 1):
        assert probes.bqa_mma_probe(kind, 152, 10, _ptr(out), torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
    assert probes.bqa_mma_probe(2, 152, 10, _ptr(out), torch.cuda.current_stream().cuda_stream) == 1
    for kind in (0, 1):
        assert 10.0 < bench.mma_peak_tflops(torch.device("cuda"), kind) < 5000.0


_MERGE_SCRIPT = """
import sys, numpy as np
from bqa_gb300 import _lib
from tests.test_gpu_kernels import random_state
from tests.test_gpu_autotune import plan_sweep
out = {}
for name, chi, prec in (("mixed_n18_chi3", 3, "single"), ("grid3x4_chi4_damped", 5, "single"),
                        ("tree9", 2, "single"), ("mixed_n18_chi3", 3, "double")):
    octx, st, job = random_state(name, chi, seed=5, precision=prec)
    key = f"{name}_{chi}_{prec}"
    for v in (_lib.BQA_VARIANT_GENERIC, _lib.BQA_VARIANT_DEFAULT):
        for two_stage in (True, False):
            out[f"{key}_plan{v}{two_stage}"] = plan_sweep(job, [v] * len(job.classes), two_stage)
            out[f"{key}_dist{v}{two_stage}"] = job.dist_parts.cpu().numpy()
    out[key + "_rho"] = job.density_matrices()
    out[key + "_zz"] = job.edge_zz()
    job.run_layer(0.07, 0.11)
    tens, msgs, lam = job.get_state()
    out[key + "_msgs"] = msgs
    out[key + "_lam"] = lam
    out[key + "_bloch"] = job.bloch_vectors()
np.savez(sys.argv[1], **out)
"""


def test_merged_class_launch_bit_identical_to_per_class(tmp_path):
    """One launch of the generic kernel over several degree classes (the default) gives the
    bits of one launch per class (BQA_GB300_MERGE_CLASSES=0): BP sweeps, extended messages,
    open-bond blocks and densities, through a whole gate layer, in both precisions."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    out = {}
    for flag in ("1", "0"):
        env = dict(os.environ, BQA_GB300_MERGE_CLASSES=flag, PYTHONPATH=str(root))
        f = tmp_path / f"merge{flag}.npz"
        subprocess.run([sys.executable, "-c", _MERGE_SCRIPT, str(f)], cwd=root, env=env, check=True, timeout=600)
        out[flag] = np.load(f)
    assert sorted(out["1"].files) == sorted(out["0"].files)
    for k in out["1"].files:
        assert np.array_equal(out["1"][k], out["0"][k]), k
        assert np.isfinite(out["1"][k]).all(), k


def test_launch_count_counts_each_kernel_launch():
    """bqa_launch_count grows by one per kernel the library launches: a densities pass of a
    single-class job is one launch, a two-stage sweep of it two (half-node kernel + combine)."""
    _, _, job = random_state("rr3_n16_chi4", 4, seed=2)
    lib = job.lib
    n0 = lib.dll.bqa_launch_count()
    job.density_matrices()
    assert lib.dll.bqa_launch_count() - n0 == 1
    n1 = lib.dll.bqa_launch_count()
    lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), 4, job.dtype, _ptr(job.msgs[0]),
             _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), None, job.stream)
    assert lib.dll.bqa_launch_count() - n1 == 2
