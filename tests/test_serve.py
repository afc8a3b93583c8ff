"""Job server: footprint admission (CPU) and, on the GPU, every job's result in a concurrent
mix equals its result alone."""
import numpy as np
import pytest

from bqa_gb300 import instances
from bqa_gb300.layout import build_context
from tests import golden_cases as gc


def small_jobs():
    jobs = [gc.config(n) for n in ("rr3_n16_chi4", "rr4_n20_chi4", "mixed_n18_chi3", "rr3_n12_measure")]
    for i, (n, d, chi) in enumerate([(400, 3, 8), (600, 4, 4), (300, 3, 4)]):
        rng = np.random.default_rng(i)
        e = instances.random_regular_edges(n, d, i)
        jobs.append(instances.qubo_config(e, 2.0 * rng.integers(0, 2, len(e)) - 1, rng.normal(0, 0.5, n),
                                          max_bond_dim=chi, bp_eps=1e-5, max_bp_iter_number=50,
                                          schedule=instances.anneal_schedule(2.0, 15)))
    return jobs


def test_footprint_grows_with_size_and_bond_dim():
    from bqa_gb300.serve import job_footprint
    a = job_footprint(build_context(instances.headline_gpu_job(n=1000, chi=4)))
    b = job_footprint(build_context(instances.headline_gpu_job(n=2000, chi=4)))
    c = job_footprint(build_context(instances.headline_gpu_job(n=1000, chi=8)))
    assert a < b < 2.2 * a and c > 4 * a


def test_too_large_job_is_rejected_at_submission():
    torch = pytest.importorskip("torch")
    from bqa_gb300.serve import JobServer
    srv = JobServer(hbm_budget=1 << 20, device="cpu")
    with pytest.raises(ValueError, match="above the server budget"):
        srv.submit(instances.headline_gpu_job(n=1000, chi=8))


@pytest.mark.gpu
@pytest.mark.timeout(600)
@pytest.mark.parametrize("pack_bp", [True, False])
def test_results_alone_equal_results_in_the_mix(pack_bp):
    """Packed (BP runs of waiting jobs swept in shared launches) or not, every job's results in
    the mix are the bits of its run alone."""
    import bqa_gb300
    from bqa_gb300.serve import JobServer, job_footprint
    jobs = small_jobs()
    alone = [bqa_gb300.run_qa(dict(j)) for j in jobs]
    fps = [job_footprint(build_context(dict(j))) for j in jobs]
    budget = sum(sorted(fps)[-3:])          # at most ~3 jobs resident: admission must queue
    srv = JobServer(hbm_budget=budget, pack_bp=pack_bp)
    ids = [srv.submit(dict(j), arrival=0.01 * k) for k, j in enumerate(jobs)]
    out = srv.run(timeout=300)
    st = srv.stats()
    srv.close()
    for i, want in zip(ids, alone):
        got = out[i]
        assert [g[0] for g in got] == [w[0] for w in want]
        for g, w in zip(got, want):
            assert np.array_equal(np.asarray(g[1]), np.asarray(w[1]))
    assert st["jobs"] == len(jobs) and st["p99_s"] >= st["p50_s"] > 0
    if pack_bp:
        assert st["bp_packing"]["packed_calls"] > 0 and st["bp_packing"]["max_runs_per_call"] >= 1
