"""Index algebra of the 2xFP16 tensor-core kernel's closing contractions, on the CPU.

bqa_gb300/csrc/tc_f16x2_d3c16.cuh writes the closing operands of a half-node from the products'
accumulators (write_block) into K-split stage buffers (x_off, r_off), the tensor cores form
D = X R^T per stage, and epilogue_block folds D into the block P.  This test restates those
index maps with numpy (each formula as the kernel writes it) and checks that every operand
element is written exactly once per stage (the padding of the strides never, and never read:
it stays NaN) and that the folded D equals
P[o][o'] = sum_kappa conj(X[o, kappa]) R[o', kappa] for the three blocks
P_0 = <V_1|V_2>, P_2 = <V_0|V_1>, P_1 = <V_0|V_2>.  The hi/lo split is modelled as exact
(hi = (1 - 2^-5) v, lo = 2^-5 v), so a misplaced hi or lo row shows as an error.
"""
import numpy as np

X_LBO, X_SBO, R_LBO, R_SBO = 1152, 144, 144, 2304
X_BYTES, R_BYTES = 16 * X_LBO, 4 * R_SBO
SPLIT = 2.0 ** -5


def x_off(m, k):   # MN-major, bytes
    return (k >> 3) * X_LBO + (m >> 3) * X_SBO + (k & 7) * 16 + (m & 7) * 2


def r_off(n, k):   # K-major, bytes
    return (n >> 3) * R_SBO + (k >> 3) * R_LBO + (n & 7) * 16 + (k & 7) * 2


def accumulator_rows(V, which):
    """Rows r = 16 hi + lo of the products' accumulator of V_which, columns 2 y + q."""
    if which == 2:
        vals = V.reshape(256, 16)                        # rows (a, b), new index c
    elif which == 1:
        vals = V.transpose(0, 2, 1).reshape(256, 16)     # rows (a, c), new index b
    else:
        vals = V.transpose(1, 2, 0).reshape(256, 16)     # rows (b, c), new index a
    f = np.empty((256, 32))
    f[:, 0::2], f[:, 1::2] = vals.real, vals.imag
    return f


def write_block(blk, Vs, bufs):
    """Both stages of block blk (stage rho into bufs[rho], arrays of 2-byte slots)."""
    fx = accumulator_rows(Vs[1 if blk == 0 else 0], 1 if blk == 0 else 0)
    fr = accumulator_rows(Vs[1 if blk == 1 else 2], 1 if blk == 1 else 2)
    for r in range(256):
        hi, lo = r >> 4, r & 15
        O, V = (lo, hi) if blk == 1 else (hi, lo)
        m0 = 16 * (O >> 2) + 4 * (O & 3)
        for rho in range(2):
            odd = (V + rho) & 1
            for i in range(8):
                x0, x1 = fx[r, 4 * i + 2 * odd], fx[r, 4 * i + 2 * odd + 1]
                k = 8 * (2 * i + odd) + (V >> 1)
                o = x_off(m0, k) // 2
                for j, v in enumerate((x0 * (1 - SPLIT), x0 * SPLIT, x1 * (1 - SPLIT), x1 * SPLIT)):
                    assert np.isnan(bufs[rho][o + j])
                    bufs[rho][o + j] = v
        U, Op = (lo, hi) if blk == 0 else (hi, lo)
        for rho in range(2):
            odd = (U + rho) & 1
            for q in range(2):
                vals = []
                for i in range(4):
                    vals += [fr[r, 8 * i + 2 * odd + q], fr[r, 8 * i + 4 + 2 * odd + q]]
                o = (X_BYTES + r_off(2 * Op + q, 8 * U)) // 2
                for e, v in enumerate(vals):
                    for part, sc in ((0, 1 - SPLIT), (1, SPLIT)):
                        idx = o + part * R_BYTES // 2 + e
                        assert np.isnan(bufs[rho][idx])
                        bufs[rho][idx] = v * sc


def stage_product(buf):
    """D[m][n] = sum_k X[m][k] (R_hi[n][k] + R_lo[n][k]) over the stage's K = 128."""
    m = np.arange(64)[:, None]
    n = np.arange(32)[:, None]
    k = np.arange(128)[None, :]
    X = buf[x_off(m, k) // 2]
    R = buf[(X_BYTES + r_off(n, k)) // 2] + buf[(X_BYTES + R_BYTES + r_off(n, k)) // 2]
    return X @ R.T


def fold(D):
    """epilogue_block: lanes 2 i + l of quarter w hold hi/lo rows of P row 8 w + i."""
    P = np.zeros((16, 16), complex)
    for w in range(4):
        g = {L: D[16 * w + L] + D[16 * w + (L ^ 1)] for L in range(16)}
        for L in range(0, 16, 2):
            pr = 8 * w + (L >> 1)
            o, p = pr >> 1, pr & 1
            own, h = g[L][0::2], g[L ^ 2][1::2]
            if p:
                P[o] += 1j * (h - own)
            else:
                P[o] += own + h
    return P


def test_closing_stages_reconstruct_the_blocks():
    rng = np.random.default_rng(0)
    Vs = [rng.normal(size=(16, 16, 16)) + 1j * rng.normal(size=(16, 16, 16)) for _ in range(3)]
    want = [np.einsum("abc,xbc->ax", Vs[1].conj(), Vs[2]),   # P_0: open a
            np.einsum("abc,abx->cx", Vs[0].conj(), Vs[1]),   # P_2: open c
            np.einsum("abc,axc->bx", Vs[0].conj(), Vs[2])]   # P_1: open b
    for blk in range(3):
        bufs = [np.full(X_BYTES // 2 + R_BYTES, np.nan) for _ in range(2)]
        write_block(blk, Vs, bufs)
        for b in bufs:   # every element written exactly once; the strides' padding stays unset (NaN)
            assert (~np.isnan(b)).sum() == 64 * 128 + 2 * 32 * 128
        P = fold(stage_product(bufs[0]) + stage_product(bufs[1]))
        assert np.abs(P - want[blk]).max() < 1e-12 * np.abs(want[blk]).max()
