"""The canonicalisation entry point that allocates nothing, checked against the regular one.

``bqa_canonicalize_noalloc`` is for callers that cannot allocate device memory -- a host
whose device heap is owned by an external pool allocator, or a pipeline that must not pay
the device-wide synchronisation of cudaMalloc/cudaFree.  It keeps its intermediate factors
in a static device array inside the library.  This test calls it through the C ABI twice in
a row (the second call sees the first call's leftovers in the shared array) and compares
canonicalisers, bond spectra and their column maxima with bqa_env_factor + bqa_bond_canon
run on caller buffers, to the kernel-test tolerance (2e-5 relative).  It sits in a file of
its own named to be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib  # noqa: E402

RTOL = 2e-5


def _random_ext_msgs(rng, E, n):
    a = rng.normal(size=(E, n, n)) + 1j * rng.normal(size=(E, n, n))
    m = a @ np.conj(np.swapaxes(a, 1, 2))
    m[:, :, n // 2:] *= 1e-3          # spread the spectrum: some small eigenvalues
    m[:, n // 2:, :] *= 1e-3
    m /= np.trace(m, axis1=1, axis2=2)[:, None, None]
    return torch.from_numpy(m.astype(np.complex64).reshape(-1)).cuda()


def _regular(lib, ext, E, n, eps, stream):
    lu = torch.empty_like(ext)
    ul = torch.empty_like(ext)
    canon = torch.empty_like(ext)
    lam = torch.empty(E // 2 * n, dtype=torch.float32, device="cuda")
    colmax = torch.zeros(n, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.call("bqa_env_factor", ext.data_ptr(), E, n, _lib.BQA_C64, eps, lu.data_ptr(), ul.data_ptr(),
             status.data_ptr(), stream)
    lib.call("bqa_bond_canon", lu.data_ptr(), ul.data_ptr(), E, n, _lib.BQA_C64, eps, canon.data_ptr(),
             lam.data_ptr(), colmax.data_ptr(), status.data_ptr(), stream)
    return canon, lam, colmax, status


def _noalloc(lib, ext, E, n, eps, stream):
    canon = torch.full_like(ext, complex(7.0, 7.0))
    lam = torch.full((E // 2 * n,), 7.0, dtype=torch.float32, device="cuda")
    colmax = torch.full((n,), 123, dtype=torch.int32, device="cuda")   # must be cleared by the call
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.call("bqa_canonicalize_noalloc", ext.data_ptr(), E, n, _lib.BQA_C64, eps, canon.data_ptr(),
             lam.data_ptr(), colmax.data_ptr(), status.data_ptr(), stream)
    return canon, lam, colmax, status


def _rel(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("E,n", [(600, 8), (200, 32)])
def test_noalloc_matches_regular_two_calls_in_a_row(E, n):
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    eps = 1e-6
    for call in range(2):
        ext = _random_ext_msgs(rng, E, n)
        want = _regular(lib, ext, E, n, eps, stream)
        got = _noalloc(lib, ext, E, n, eps, stream)
        torch.cuda.synchronize()
        assert int(got[3].item()) == int(want[3].item()) == 0
        assert _rel(got[0], want[0]) < RTOL, f"canonicalisers differ on call {call}"
        assert _rel(got[1], want[1]) < RTOL, f"lambdas differ on call {call}"
        assert np.allclose(got[2].view(torch.float32).cpu().numpy(), want[2].view(torch.float32).cpu().numpy(),
                           rtol=RTOL, atol=0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    E, n = 8192, 32             # 2 * 8192 * 1024 * 8 B = 128 MiB > 64 MiB
    dummy = torch.empty(1, dtype=torch.complex64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.BqaError, match="static scratch"):
        lib.call("bqa_canonicalize_noalloc", dummy.data_ptr(), E, n, _lib.BQA_C64, 1e-6, dummy.data_ptr(),
                 dummy.data_ptr(), dummy.data_ptr(), status.data_ptr(), stream)
