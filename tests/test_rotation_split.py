"""The exact BF16 digit splitting behind the tensor-core restart rotation
(severo.jl_gb300/csrc/sv_rotate_tc.cu), emulated on the CPU.

The kernel computes W P (W: rows of double-float values, P: FP64) as sums of
BF16 GEMMs: every row of W and every column of P is scaled by a power of two
and cut into six balanced 8-bit digits; the products of slices s, t with the
same level L = s + t are summed in one FP32 accumulator, and the levels are
recombined by Horner.  These tests restate the cutting with the kernel's
arithmetic (FP32 two-sum steps for W, exact FP64 steps for P) and check the
properties its exactness rests on: digits are integers in [-128, 128] (exact
in BF16), every level sum is an integer below 2^23 (exact in FP32 whatever the
order of accumulation), and the recombined product agrees with the exact one
to the double-float level (2^-46 of the row and column scales).
"""
import numpy as np

SLICES = 6


def _two_sum(a, b):
    s = np.float32(a + b)
    v = np.float32(s - a)
    e = np.float32(np.float32(a - np.float32(s - v)) + np.float32(b - v))
    return s, e


def cut_rows(wh, wl):
    """Rows of a double-float matrix (hi, lo FP32, shape m x k) -> (exponents
    e_i, digits a[s] of shape m x k), as the kernel's threads cut them."""
    wh = wh.astype(np.float32)
    wl = wl.astype(np.float32)
    mx = np.abs(wh).max(axis=1)
    e = np.where(mx > 0, np.floor(np.log2(np.maximum(mx, np.float32(1e-30)))).astype(np.int64) + 1, 0)
    sc = np.ldexp(np.float32(128.0), -e).astype(np.float32)[:, None]
    rh = (wh * sc).astype(np.float32)          # exact: power-of-two scaling
    rl = (wl * sc).astype(np.float32)
    digits = []
    for _ in range(SLICES):
        d = np.rint(rh).astype(np.float32)
        digits.append(d)
        u = np.float32(rh - d)
        rh, rl = _two_sum(u, rl)
        rh = np.float32(rh * 256)
        rl = np.float32(rl * 256)
    return e, np.stack(digits)


def cut_cols(p):
    """Columns of an FP64 matrix (k x n) -> (exponents f_c, digits b[t] k x n)."""
    mx = np.abs(p).max(axis=0)
    f = np.where(mx > 0, np.floor(np.log2(np.maximum(mx, 1e-300))).astype(np.int64) + 1, 0)
    rem = np.ldexp(p, -f[None, :]) * 128.0
    digits = []
    for _ in range(SLICES):
        d = np.rint(rem)
        digits.append(d)
        rem = (rem - d) * 256.0
    return f, np.stack(digits)


def split_product(wh, wl, p):
    e, a = cut_rows(wh, wl)
    f, b = cut_cols(p)
    levels = []
    for L in range(SLICES):
        acc = np.zeros((wh.shape[0], p.shape[1]))
        for s in range(SLICES):
            t = L - s
            if 0 <= t < SLICES:
                acc += a[s].astype(np.float64) @ b[t].astype(np.float64)   # integer products, exact
        levels.append(acc)
    val = levels[SLICES - 1]
    for L in range(SLICES - 2, -1, -1):
        val = val * 2.0 ** -8 + levels[L]
    out = np.ldexp(val, (e[:, None] + f[None, :] - 14))
    return out, a, b, levels, e, f


def _basis(rng, m, k):
    q, _ = np.linalg.qr(rng.standard_normal((m, k)))
    wh = q.astype(np.float32)
    wl = (q - wh.astype(np.float64)).astype(np.float32)
    return wh, wl, wh.astype(np.float64) + wl.astype(np.float64)


def test_digits_are_bf16_integers_and_levels_exact():
    rng = np.random.default_rng(11)
    wh, wl, _ = _basis(rng, 3000, 57)
    p, _ = np.linalg.qr(rng.standard_normal((57, 50)))
    _, a, b, levels, _, _ = split_product(wh, wl, p)
    for d in (a, b):
        assert np.all(d == np.rint(d)) and np.abs(d).max() <= 128
    # every level sum is an integer below 2^23: exact in an FP32 accumulator
    for acc in levels:
        assert np.all(acc == np.rint(acc)) and np.abs(acc).max() < 2 ** 23


def test_recombined_product_at_double_float_accuracy():
    rng = np.random.default_rng(12)
    for m, k, n in [(2000, 57, 50), (500, 9, 2), (128, 64, 64)]:
        wh, wl, w = _basis(rng, m, k)
        p = rng.standard_normal((k, n))
        out, *_ = split_product(wh, wl, p)
        exact = w @ p
        scale = np.abs(w).max(axis=1)[:, None] * np.abs(p).max(axis=0)[None, :] * k
        assert np.all(np.abs(out - exact) <= 2.0 ** -46 * scale)


def test_zero_rows_and_columns():
    rng = np.random.default_rng(13)
    wh, wl, w = _basis(rng, 256, 20)
    wh[5] = 0
    wl[5] = 0
    w[5] = 0
    p = rng.standard_normal((20, 7))
    p[:, 3] = 0
    out, *_ = split_product(wh, wl, p)
    assert np.all(out[5] == 0) and np.all(out[:, 3] == 0)
    exact = w @ p
    assert np.abs(out - exact).max() <= 2.0 ** -44 * np.abs(exact).max()
