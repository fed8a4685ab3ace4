"""CPU restatement of the exact-digit tensor-core products
(nuclearcgm_gb300/csrc/k_tcgram_exact.cu): the digit split, the exact level
sums and their 64-bit combination, and the shared-memory addressing of the
stacked B digit planes. The GPU kernels are tested against numpy in
tests/test_gpu_tcgram.py; this checks the arithmetic they rely on."""
import numpy as np

K_DIG = 6
K_SBO, K_LBO = 512, 128          # core matrices: 8 rows x 16 bytes, K 32
K_ABYTES, K_BBYTES = 128 * 32 * 2, 64 * 32 * 2


def scaled_int(x, e):
    """round(x 2^(42 - e)), half away from zero (scaledInt)."""
    w = np.floor(np.abs(x) * 2.0 ** (42 - e) + 0.5).astype(np.int64)
    return np.where(x < 0, -w, w)


def digits(w):
    """The six signed digits a_t with w = sum_t a_t 2^(35 - 7t) (digits()):
    one 21-bit rounding split, then three digits from each half."""
    w = np.asarray(w, np.int64)
    hh = (w + (1 << 20)) >> 21
    lo = w - (hh << 21)
    hi = hh.copy()
    d = [None] * 6
    for t in range(2):
        sh = 14 - 7 * t
        a = (hi + (1 << (sh - 1))) >> sh
        d[t] = a
        hi = hi - (a << sh)
        b = (lo + (1 << (sh - 1))) >> sh
        d[3 + t] = b
        lo = lo - (b << sh)
    d[2], d[5] = hi, lo
    return np.stack(d, -1)


def off16(row, k):
    """Byte offset of element (row, k) in a K-major tile of core matrices."""
    return (row >> 3) * K_SBO + (k >> 3) * K_LBO + (row & 7) * 16 + (k & 7) * 2


def exact_gram(S, T, fold_rows=256):
    """S^T T for real blocks through the digit products: per-column power of
    two scales, level sums per fold block (checked exact in FP32), the
    64-bit combination, one conversion per entry."""
    es = np.frexp(np.abs(S).max(0))[1]
    et = np.frexp(np.abs(T).max(0))[1]
    ds = digits(scaled_int(S, es[None, :]))   # (N, p, 6)
    dt = digits(scaled_int(T, et[None, :]))
    acc = np.zeros((S.shape[1], T.shape[1]), dtype=object)
    for r0 in range(0, S.shape[0], fold_rows):
        sl = slice(r0, r0 + fold_rows)
        total = np.zeros(acc.shape, dtype=object)
        for lev in range(K_DIG):
            L = sum(ds[sl, :, t].T @ dt[sl, :, lev - t]
                    for t in range(lev + 1))
            assert np.abs(L).max() < 2 ** 24   # exact in an FP32 accumulator
            total = total * 128 + L.astype(object)
        assert max(abs(v) for v in total.ravel()) < 2.0 ** 58.1
        acc = acc + total
    out = np.array([[float(v) for v in row] for row in acc])
    return out * 2.0 ** (es[:, None] + et[None, :] - 7 * (K_DIG + 1))


def test_digit_split_is_exact_and_bounded():
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 20000) * 2.0 ** rng.integers(-30, 0, 20000)
    e = np.frexp(np.abs(x).max())[1]
    w = scaled_int(x, e)
    d = digits(w)
    assert np.abs(d[:, 0]).max() <= 128 and np.abs(d[:, 1:]).max() <= 64
    back = sum(d[:, t] << (35 - 7 * t) for t in range(K_DIG))
    assert np.array_equal(back, w)
    # the split loses below 2^-42 of the column scale
    assert np.abs(w * 2.0 ** (e - 42) - x).max() <= 2.0 ** (e - 43)


def test_level_sums_exact_and_gram_accurate():
    rng = np.random.default_rng(2)
    N, p, q = 700, 6, 5
    S = rng.normal(size=(N, p))
    T = rng.normal(size=(N, q))
    S[:, 0] *= 1e-6                      # a column far below the others
    ref = S.T @ T
    C = exact_gram(S, T)
    scale = np.outer(np.linalg.norm(S, axis=0), np.linalg.norm(T, axis=0))
    assert (np.abs(C - ref) / scale).max() < 1e-12


def test_worst_case_digits_keep_level_sums_below_fp32_range():
    """All digits at their bounds with one sign: 256-row level sums stay
    below 2^24 and the 16-block 64-bit sum below 2^63."""
    a = np.array([128] + [64] * 5, np.int64)
    levels = [sum(int(a[t]) * int(a[lev - t]) for t in range(lev + 1)) * 256
              for lev in range(K_DIG)]
    assert max(levels) < 2 ** 24
    fold = sum(L * 128 ** (K_DIG - 1 - lev) for lev, L in enumerate(levels))
    assert 16 * fold < 2 ** 63


def test_stacked_b_planes_read_as_one_operand():
    """Digit plane u of a 64-row B tile starts 4 KB = 8 row groups after
    plane u - 1, so planes u0..u1 read as one N = 64 (u1 - u0 + 1) operand:
    row 64 u + j of the stacked operand is row j of plane u."""
    assert K_BBYTES == 8 * K_SBO
    j = np.arange(64)[:, None]
    k = np.arange(32)[None, :]
    for u in range(4):
        assert np.array_equal(off16(64 * u + j, k), u * K_BBYTES + off16(j, k))
    # the half (nt & 1) of a 128-row digit tile is the same 64-row layout
    assert np.array_equal(off16(64 + j, k), K_BBYTES + off16(j, k))
