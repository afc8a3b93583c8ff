"""The canonicalisation entry point that allocates nothing, checked against the regular one.

``bqa_canonicalize_noalloc`` is for callers that cannot allocate device memory -- a host
whose device heap is owned by an external pool allocator, or a pipeline that must not pay
the device-wide synchronisation of cudaMalloc/cudaFree.  It keeps its intermediate factors
in a static device array inside the library.  This test calls it through the C ABI twice in
a row (the second call sees the first call's leftovers in the shared array) and compares
canonicalisers, bond spectra and their column maxima with bqa_env_factor + bqa_bond_canon
run on caller buffers, to the kernel-test tolerance (2e-5 relative in complex64, 1e-12 in
complex128).  One case makes the first call larger than the second, so the second call's
factors start inside the first call's leftovers at a different stride.  It sits in a file of
its own named to be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from bqa_gb300 import _lib  # noqa: E402

RTOL = {_lib.BQA_C64: 2e-5, _lib.BQA_C128: 1e-12}
CTYPE = {_lib.BQA_C64: (np.complex64, torch.float32, torch.int32),
         _lib.BQA_C128: (np.complex128, torch.float64, torch.int64)}


def _random_ext_msgs(rng, E, n, dtype):
    a = rng.normal(size=(E, n, n)) + 1j * rng.normal(size=(E, n, n))
    m = a @ np.conj(np.swapaxes(a, 1, 2))
    m[:, :, n // 2:] *= 1e-3          # spread the spectrum: some small eigenvalues
    m[:, n // 2:, :] *= 1e-3
    m /= np.trace(m, axis1=1, axis2=2)[:, None, None]
    return torch.from_numpy(m.astype(CTYPE[dtype][0]).reshape(-1)).cuda()


def _regular(lib, ext, E, n, eps, dtype, stream):
    _, real, bits = CTYPE[dtype]
    lu = torch.empty_like(ext)
    ul = torch.empty_like(ext)
    canon = torch.empty_like(ext)
    lam = torch.empty(E // 2 * n, dtype=real, device="cuda")
    colmax = torch.zeros(n, dtype=bits, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.call("bqa_env_factor", ext.data_ptr(), E, n, dtype, eps, lu.data_ptr(), ul.data_ptr(),
             status.data_ptr(), stream)
    lib.call("bqa_bond_canon", lu.data_ptr(), ul.data_ptr(), E, n, dtype, eps, canon.data_ptr(),
             lam.data_ptr(), colmax.data_ptr(), status.data_ptr(), stream)
    return canon, lam, colmax.view(real), status


def _noalloc(lib, ext, E, n, eps, dtype, stream):
    _, real, bits = CTYPE[dtype]
    canon = torch.full_like(ext, complex(7.0, 7.0))
    lam = torch.full((E // 2 * n,), 7.0, dtype=real, device="cuda")
    colmax = torch.full((n,), 123, dtype=bits, device="cuda")   # must be cleared by the call
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.call("bqa_canonicalize_noalloc", ext.data_ptr(), E, n, dtype, eps, canon.data_ptr(),
             lam.data_ptr(), colmax.data_ptr(), status.data_ptr(), stream)
    return canon, lam, colmax.view(real), status


def _rel(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("dtype,sizes", [
    (_lib.BQA_C64, [(600, 8), (600, 8)]),
    (_lib.BQA_C64, [(200, 32), (200, 32)]),
    (_lib.BQA_C64, [(600, 32), (200, 8)]),      # second call inside the first call's leftovers
    (_lib.BQA_C128, [(300, 16), (100, 8)]),
])
def test_noalloc_matches_regular_two_calls_in_a_row(dtype, sizes):
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    eps = 1e-6
    rtol = RTOL[dtype]
    for call, (E, n) in enumerate(sizes):
        ext = _random_ext_msgs(rng, E, n, dtype)
        want = _regular(lib, ext, E, n, eps, dtype, stream)
        got = _noalloc(lib, ext, E, n, eps, dtype, stream)
        torch.cuda.synchronize()
        assert int(got[3].item()) == int(want[3].item()) == 0
        assert _rel(got[0], want[0]) < rtol, f"canonicalisers differ on call {call}"
        assert _rel(got[1], want[1]) < rtol, f"lambdas differ on call {call}"
        assert np.allclose(got[2].cpu().numpy(), want[2].cpu().numpy(), rtol=rtol, atol=0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    E, n = 8192, 32             # 2 * 8192 * 1024 * 8 B = 128 MiB > 64 MiB
    dummy = torch.empty(1, dtype=torch.complex64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.BqaError, match="static scratch"):
        lib.call("bqa_canonicalize_noalloc", dummy.data_ptr(), E, n, _lib.BQA_C64, 1e-6, dummy.data_ptr(),
                 dummy.data_ptr(), dummy.data_ptr(), status.data_ptr(), stream)
    with pytest.raises(_lib.BqaError, match="odd number"):
        lib.call("bqa_canonicalize_noalloc", dummy.data_ptr(), 201, 8, _lib.BQA_C64, 1e-6, dummy.data_ptr(),
                 dummy.data_ptr(), dummy.data_ptr(), status.data_ptr(), stream)
