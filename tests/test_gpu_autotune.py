"""The autotuner's search space and its plans, on the GPU.

Every BP-sweep variant bqa_bp_sweep_plan offers (register-tiled or generic message kernel per
degree class, two-stage or one-stage sweep) computes one oracle BP sweep to the complex64
kernel tolerance (2e-5 relative); a plan of DEFAULT variants launches exactly what the
unplanned entry points launch (bit-identical); a tuned anneal stays within the complex64
end-to-end tolerance of the FP64 oracle and runs the same steps through the native driver,
the graph-replayed BP runs and the launch-by-launch Python driver with identical state.
"""
import ctypes

import numpy as np
import pytest

from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib, autotune  # noqa: E402
from bqa_gb300.engine import Annealer, _ptr  # noqa: E402
from bqa_gb300.layout import build_context  # noqa: E402
from oracle import bqa_oracle as orc  # noqa: E402
from tests.test_gpu_kernels import RTOL, random_state, rel_err  # noqa: E402

V = _lib
CASES = [("rr3_n16_chi4", 4), ("rr3_n24_chi8", 8), ("rr3_n16_chi4", 16), ("rr4_n20_chi4", 4),
         ("rr4_n20_chi4", 8), ("mixed_n18_chi3", 3), ("mixed_n18_chi3", 4), ("grid3x4_chi4_damped", 12)]


def oracle_sweep(octx, st):
    want = np.empty_like(st.msgs)
    for d, t in st.degree_to_tensor.items():
        L = octx.degree_to_layout[d]
        for mm, p in zip(orc.pass_msgs(t, [st.msgs[p] for p in L.input_msgs_position]), L.output_msgs_position):
            want[p] = mm
    return want


def plan_sweep(job, variants, two_stage):
    arr = (ctypes.c_int32 * len(variants))(*variants)
    job.dist_parts.zero_()
    job.lib.call("bqa_bp_sweep_plan", job._class_array(), len(job.classes), job.chis, job.dtype, arr,
                 _ptr(job.msgs[0]), _ptr(job.msgs[1]), _ptr(job.lu) if two_stage else None, job.E,
                 _ptr(job.dist_parts), None, job.stream)
    return job.msgs[1][: job.E * job.chis * job.chis].cpu().numpy().reshape(job.E, job.chis, job.chis)


@pytest.mark.parametrize("name,chi", CASES)
@pytest.mark.parametrize("two_stage", [True, False])
@pytest.mark.parametrize("variant", [V.BQA_VARIANT_TILED, V.BQA_VARIANT_GENERIC])
def test_every_variant_matches_oracle(name, chi, two_stage, variant):
    octx, st, job = random_state(name, chi, seed=4)
    want = oracle_sweep(octx, st)
    variants = [variant] * len(job.classes)
    try:
        got = plan_sweep(job, variants, two_stage)
    except _lib.BqaError as e:
        assert variant == V.BQA_VARIANT_TILED and "register-tiled" in str(e)
        return
    assert rel_err(got, want) < RTOL
    num, den = job.dist_parts.view(torch.int32)[:2].view(torch.float32).cpu().numpy()
    d_want = orc.get_dist(want, st.msgs)
    assert abs(np.sqrt(num) / np.sqrt(den) - d_want) < 1e-5 * max(1.0, d_want)


@pytest.mark.parametrize("name,chi", [("rr3_n16_chi4", 16), ("mixed_n18_chi3", 4), ("rr4_n20_chi4", 8)])
def test_default_plan_is_the_unplanned_sweep(name, chi):
    octx, st, job = random_state(name, chi, seed=5)
    for two_stage in (True, False):
        got = plan_sweep(job, [V.BQA_VARIANT_DEFAULT] * len(job.classes), two_stage)
        job.dist_parts.zero_()
        if two_stage:
            job.lib.call("bqa_bp_sweep_split", job._class_array(), len(job.classes), chi, job.dtype,
                         _ptr(job.msgs[0]), _ptr(job.msgs[1]), _ptr(job.lu), job.E, _ptr(job.dist_parts), None,
                         job.stream)
        else:
            job.lib.call("bqa_bp_sweep", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job.msgs[0]),
                         _ptr(job.msgs[1]), _ptr(job.dist_parts), None, job.stream)
        ref = job.msgs[1][: got.size].cpu().numpy().reshape(got.shape)
        assert np.array_equal(got, ref)


def test_tuned_anneal_matches_oracle_and_every_driver():
    autotune.clear_cache()
    name = "rr3_n24_chi8"
    conf = gc.config(name)
    ctx = build_context(dict(conf))
    steps = [i for i in ctx.instructions if isinstance(i, dict)]
    jobs = {"graph": Annealer(ctx, autotune=True, graphs=True),
            "native": Annealer(ctx, autotune=True, graphs=False),
            "python": Annealer(ctx, autotune=True, native=False)}
    for ins in steps:
        for job in jobs.values():
            job.run_layer(ins["xtime"], ins["ztime"])
    g = jobs["graph"]
    assert g.plans, "the tuner made no plan"
    for p in g.plans.values():
        assert len(p.variants) == len(g.classes)
        assert all(v in (V.BQA_VARIANT_DEFAULT, V.BQA_VARIANT_TILED, V.BQA_VARIANT_GENERIC, V.BQA_VARIANT_TENSOR)
                   for v in p.variants)
        assert p.describe()["form"] in ("two-stage", "one-stage")
    # all three drivers ran the same plans: identical state
    ref = g.get_state()
    for other in ("native", "python"):
        got = jobs[other].get_state()
        assert jobs[other].stats == g.stats
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
        for d in ref[0]:
            assert np.array_equal(got[0][d], ref[0][d])
    want = gc.arrays(name)["result0_bloch_vectors"]
    err = np.abs(g.bloch_vectors() - want).max()
    assert err < 1e-3, err


@pytest.mark.parametrize("name,chi", [("mixed_n18_chi3", 3), ("rr4_n20_chi4", 4), ("grid3x4_chi4_damped", 5),
                                      ("rr3_n24_chi8", 8), ("mixed_n18_chi3", 4)])
@pytest.mark.parametrize("two_stage", [True, False])
def test_generic_cta_size_gives_the_same_messages(name, chi, two_stage):
    """The generic kernel at 2, 16 or 32 warps per node writes the bits of its own CTA size,
    and equals the oracle; above 8 warps bond dims beyond 8 are refused."""
    from bqa_gb300.autotune import generic_warps
    octx, st, job = random_state(name, chi, seed=4)
    want = oracle_sweep(octx, st)
    ref = plan_sweep(job, [V.BQA_VARIANT_GENERIC] * len(job.classes), two_stage)
    assert rel_err(ref, want) < RTOL
    for w in (2, 16, 32):
        got = plan_sweep(job, [generic_warps(w)] * len(job.classes), two_stage)
        assert np.array_equal(got, ref), w


def test_generic_cta_size_above_8_warps_refused_beyond_bond_dim_8():
    from bqa_gb300.autotune import generic_warps
    _, _, job = random_state("rr3_n16_chi4", 12, seed=4)
    with pytest.raises(_lib.BqaError, match="no 512-thread build"):
        plan_sweep(job, [generic_warps(16)] * len(job.classes), True)
    with pytest.raises(_lib.BqaError, match="unknown variant"):
        plan_sweep(job, [V.BQA_VARIANT_TILED | (4 << 8)] * len(job.classes), True)
