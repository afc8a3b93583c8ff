"""Environment factors of real saturated-state messages, QR-preconditioned Jacobi vs the direct
Jacobi vs FP64 eigen-decomposition.

The extended messages of a 200-node 3-regular anneal at bond dim 16 (the headline workload's
generator) have spectra over many decades, the case the preconditioner is for.  Both kernel
forms run in child processes (the form is fixed when the library loads); each must rebuild the
masked message (lu^H lu = sum over kept eigenpairs of lambda v v^H) to 2e-5 of its largest
entry, keep the same eigen-directions as FP64 (the projector ul lu) to 5e-3 wherever the kept
counts agree, agree on the kept count for >= 99% of messages, and the preconditioned form's
median projector error must be no worse than 1.5x the direct form's.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r"""
import sys
import numpy as np
import torch
from bqa_gb300 import instances
from bqa_gb300.engine import Annealer, _ptr
from bqa_gb300.layout import build_context
ctx = build_context(instances.headline_gpu_job(n=200, seed=0, chi=16))
steps = [i for i in ctx.instructions if isinstance(i, dict)]
job = Annealer(ctx, graphs=False)
s = 0
while job.bond_dim < 16 or s < 70:
    job.run_layer(steps[s]["xtime"], steps[s]["ztime"])
    s += 1
chi, E = job.chis, ctx.edges_number
n = 2 * chi
lib, st = job.lib, job.stream
lib.call("bqa_ext_msgs", job._class_array(), len(job.classes), chi, job.dtype, _ptr(job._msgs_cur()), _ptr(job.ext),
         float(steps[s]["ztime"]), st)
job.status.zero_()
lib.call("bqa_env_factor", _ptr(job.ext), E, n, job.dtype, float(ctx.pinv_eps), _ptr(job.lu), _ptr(job.ul),
         _ptr(job.status), st)
torch.cuda.synchronize()
k = E * n * n
np.savez(sys.argv[1], ext=job.ext[:k].cpu().numpy().reshape(E, n, n), lu=job.lu[:k].cpu().numpy().reshape(E, n, n),
         ul=job.ul[:k].cpu().numpy().reshape(E, n, n), status=int(job.status.item()), eps=float(ctx.pinv_eps))
"""


def run_form(tmp_path, qr: str) -> dict:
    env = dict(os.environ, BQA_GB300_JACOBI_QR=qr, PYTHONPATH=str(ROOT))
    f = tmp_path / f"env_qr{qr}.npz"
    subprocess.run([sys.executable, "-c", SCRIPT, str(f)], cwd=ROOT, env=env, check=True, timeout=900)
    with np.load(f) as z:
        return {k: z[k] for k in z.files}


def quality(r: dict) -> dict:
    m = r["ext"].astype(np.complex128)
    lu, ul = r["lu"].astype(np.complex128), r["ul"].astype(np.complex128)
    eps = float(r["eps"])
    w, u = np.linalg.eigh(m)
    kref = w > eps
    m_kept = np.einsum("eik,ek,ejk->eij", u, np.where(kref, w, 0.0), np.conj(u))
    recon = np.conj(np.swapaxes(lu, 1, 2)) @ lu
    rec_err = np.abs(recon - m_kept).max() / np.abs(m).max()
    kept = np.sum(np.linalg.norm(lu, axis=2) > 0, axis=1)
    same = kept == kref.sum(axis=1)
    proj = ul @ lu
    proj_ref = np.einsum("eik,ek,ejk->eij", u, kref.astype(float), np.conj(u))
    perr = np.abs(proj - proj_ref).reshape(len(m), -1).max(axis=1)[same]
    return {"rec": float(rec_err), "same": float(same.mean()), "pmax": float(perr.max()),
            "pmed": float(np.median(perr)), "status": int(r["status"])}


def test_qr_preconditioned_env_factors_match_fp64(tmp_path):
    q = quality(run_form(tmp_path, "1"))
    d = quality(run_form(tmp_path, "0"))
    print(f"QR-preconditioned: {q}\ndirect: {d}")
    for r in (q, d):
        assert r["status"] == 0
        assert r["rec"] < 2e-5
        assert r["same"] >= 0.99
        assert r["pmax"] < 5e-3
    assert q["pmed"] <= 1.5 * d["pmed"] + 1e-7


def test_qr_env_factors_with_negligible_columns_stay_finite():
    """Hermitian PSD matrices whose spectra include directions of size ~1e-20 next to O(1)
    ones (column remainders far below float32 resolution, the case whose Householder scale
    once overflowed): the factors stay finite and rebuild the masked matrix."""
    import torch
    from bqa_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(3)
    count, n, big = 256, 32, 12
    # block-diagonal: a 12x12 PSD block of O(1) eigenvalues and a 20x20 PSD block of size
    # ~1e-22, rows and columns interleaved by a random permutation: after 12 Householder steps
    # the trailing column norms are ~1e-21, representable but far below float32 resolution
    m = np.zeros((count, n, n), dtype=np.complex128)
    for e in range(count):
        x = rng.normal(size=(big, big)) + 1j * rng.normal(size=(big, big))
        y = rng.normal(size=(n - big, n - big)) + 1j * rng.normal(size=(n - big, n - big))
        blk = np.zeros((n, n), dtype=np.complex128)
        xx = x @ np.conj(x.T) + big * np.eye(big)      # kept eigenvalues well above the 1e-6 mask
        blk[:big, :big] = xx / np.trace(xx).real
        blk[big:, big:] = 1e-22 * (y @ np.conj(y.T)) / (n - big)
        p_ = rng.permutation(n)
        m[e] = blk[np.ix_(p_, p_)]
    m = m.astype(np.complex64)
    dev = torch.device("cuda")
    mt = torch.from_numpy(m.reshape(-1)).to(dev)
    lu = torch.empty_like(mt)
    ul = torch.empty_like(mt)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    lib.call("bqa_env_factor", mt.data_ptr(), count, n, _lib.BQA_C64, 1e-6, lu.data_ptr(), ul.data_ptr(),
             status.data_ptr(), st)
    torch.cuda.synchronize()
    lu_h = lu.cpu().numpy().reshape(count, n, n).astype(np.complex128)
    ul_h = ul.cpu().numpy().reshape(count, n, n).astype(np.complex128)
    assert np.isfinite(lu_h).all() and np.isfinite(ul_h).all()
    assert int(status.item()) == 0
    w, u = np.linalg.eigh(m.astype(np.complex128))
    kept = np.einsum("eik,ek,ejk->eij", u, np.where(w > 1e-6, w, 0.0), np.conj(u))
    recon = np.conj(np.swapaxes(lu_h, 1, 2)) @ lu_h
    assert np.abs(recon - kept).max() < 2e-5 * np.abs(m).max()
    assert (np.sum(np.linalg.norm(lu_h, axis=2) > 0, axis=1) == (w > 1e-6).sum(axis=1)).all()
