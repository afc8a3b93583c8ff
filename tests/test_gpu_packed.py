"""Packed BP runs (bqa_gate_layer / bqa_bp_begin / bqa_bp_packed / bqa_bp_end): several jobs'
BP loops swept in shared launches give every job the bits of its own BP run -- messages,
sweep count, exhaustion flag -- for register-tiled half-node classes shared by two jobs,
generic classes of mixed degrees, classes beyond shared memory (global-memory kernel, one
class at a time), a damped run, bond dim 16, and complex128 one-stage sweeps."""
import ctypes

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib  # noqa: E402
from tests.test_gpu_kernels import random_state  # noqa: E402

SINGLE = [("rr3_n16_chi4", 4, 1), ("rr3_n24_chi8", 4, 2), ("mixed_n18_chi3", 3, 3), ("grid3x4_chi4_damped", 4, 4),
          ("mixed_n18_chi3", 4, 5), ("rr3_n16_chi4", 16, 6), ("rr3_n24_chi8", 8, 7)]
DOUBLE = [("rr3_n16_chi4", 4, 1), ("mixed_n18_chi3", 3, 3), ("grid3x4_chi4_damped", 5, 4)]


def solo(cases, precision):
    out = []
    for name, chi, seed in cases:
        _, _, job = random_state(name, chi, seed=seed, precision=precision)
        sweeps = job.run_bp()
        out.append((job._msgs_cur()[: job.E * job.chis ** 2].cpu().numpy(), sweeps))
    return out


def packed(cases, precision, sweeps_per_call=3):
    jobs = [random_state(name, chi, seed=seed, precision=precision)[2] for name, chi, seed in cases]
    lib = jobs[0].lib
    st = torch.cuda.current_stream().cuda_stream
    structs = [j._job_struct() for j in jobs]          # (struct, class array) kept alive here
    infos = [_lib.BqaLayerInfo() for _ in jobs]
    for s, _ in structs:
        lib.call("bqa_bp_begin", ctypes.byref(s), st)
    ls_dev = torch.zeros(8 * 64, dtype=torch.int32, device="cuda")
    ls_host = (ctypes.c_int32 * (8 * 64))()
    active = list(range(len(jobs)))
    calls = 0
    while active:
        arr = (ctypes.POINTER(_lib.BqaJob) * len(active))(*[ctypes.pointer(structs[i][0]) for i in active])
        lib.call("bqa_bp_packed", arr, len(active), sweeps_per_call, ls_dev.data_ptr(), ls_host, st)
        calls += 1
        assert calls < 100
        still = []
        for k, i in enumerate(active):
            ls = (ctypes.c_int32 * 8)(*ls_host[8 * k: 8 * k + 8])
            if ls[0]:
                lib.call("bqa_bp_end", ctypes.byref(structs[i][0]), ls, ctypes.byref(infos[i]))
            else:
                still.append(i)
        active = still
    out = []
    for job, (s, _), info in zip(jobs, structs, infos):
        job.mcur = s.mcur
        out.append((job._msgs_cur()[: job.E * job.chis ** 2].cpu().numpy(), info.sweeps, info.bp_exhausted))
    return out


@pytest.mark.parametrize("precision,cases", [("single", SINGLE), ("double", DOUBLE)])
def test_packed_bp_runs_bit_identical_to_own_runs(precision, cases):
    want = solo(cases, precision)
    got = packed(cases, precision)
    for (name, chi, _), (wm, ws), (gm, gs, _) in zip(cases, want, got):
        assert gs == ws, (name, chi)
        assert np.array_equal(gm, wm), (name, chi)
        assert np.isfinite(gm).all()


def test_packed_bp_rejects_mixed_dtypes_and_bad_counts():
    a = random_state("rr3_n16_chi4", 4, seed=1, precision="single")[2]
    b = random_state("rr3_n16_chi4", 4, seed=1, precision="double")[2]
    sa, sb = a._job_struct(), b._job_struct()
    ls_dev = torch.zeros(8 * 64, dtype=torch.int32, device="cuda")
    ls_host = (ctypes.c_int32 * (8 * 64))()
    st = torch.cuda.current_stream().cuda_stream
    arr = (ctypes.POINTER(_lib.BqaJob) * 2)(ctypes.pointer(sa[0]), ctypes.pointer(sb[0]))
    with pytest.raises(_lib.BqaError, match="different dtypes"):
        a.lib.call("bqa_bp_packed", arr, 2, 1, ls_dev.data_ptr(), ls_host, st)
    with pytest.raises(_lib.BqaError, match="bad argument"):
        a.lib.call("bqa_bp_packed", arr, 0, 1, ls_dev.data_ptr(), ls_host, st)
    ls = (ctypes.c_int32 * 8)()
    with pytest.raises(_lib.BqaError, match="not done"):
        a.lib.call("bqa_bp_end", ctypes.byref(sa[0]), ls, ctypes.byref(_lib.BqaLayerInfo()))


def test_gate_layer_then_packed_bp_equals_run_layer():
    """A whole step: bqa_gate_layer + packed BP against bqa_run_layer, on two jobs."""
    from bqa_gb300.serve import BpPacker
    cases = [("rr3_n24_chi8", 8, 2), ("mixed_n18_chi3", 4, 5)]
    ref, got = [], []
    for name, chi, seed in cases:
        _, _, job = random_state(name, chi, seed=seed)
        job.run_layer(0.07, 0.11)
        tens, msgs, lam = job.get_state()
        ref.append((tens, msgs, lam, job.stats[-1]))
    packer = BpPacker()
    import threading
    jobs = [random_state(name, chi, seed=seed)[2] for name, chi, seed in cases]
    errs = []

    def step(job):
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                job.run_layer_packed(0.07, 0.11, packer)
                torch.cuda.current_stream().synchronize()
        except BaseException as e:   # noqa: BLE001
            errs.append(e)
    ts = [threading.Thread(target=step, args=(j,), daemon=True) for j in jobs]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    packer.close()
    assert not errs, errs
    for job, (tens, msgs, lam, info) in zip(jobs, ref):
        t2, m2, l2 = job.get_state()
        assert job.stats[-1] == info
        assert np.array_equal(m2, msgs) and np.array_equal(l2, lam)
        for d in tens:
            assert np.array_equal(t2[d], tens[d])
