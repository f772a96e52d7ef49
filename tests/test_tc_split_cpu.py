"""CPU restatement of the tensor-core stage GEMM's split product.

The linear engine's tensor-core mode (bacon_gb300/csrc/linear_tc.cuh) cuts
every row of A and every stage vector into five 8-bit integer slices relative
to the largest entry's power of two.  It sums the 15 slice pairs of the five
leading diagonals in eight FP32 accumulators (one per pair on diagonals 0-2,
one per diagonal for 3 and 4), in the kernel's order: K steps of 16, and
within a step the pairs with s ascending, then t ascending.  It then combines
them as integers.  This test restates that arithmetic in numpy, FP32
rounding included, and checks the properties the kernel relies on:
  - the accumulators of diagonals 0-2 stay exact FP32 integers (< 2^24);
  - the split product is within 2^-37 * K * max|a| * max|y| of the FP64
    product;
  - zero rows and zero columns give exact zeros.
"""
import numpy as np

NS, B, FB = 5, 8, 40
ACC = {(s, t): (0 if s + t == 0 else 1 + s if s + t == 1 else 3 + s if s + t == 2 else 6 if s + t == 3 else 7)
       for s in range(NS) for t in range(NS - s)}
DIAG = [0, 1, 1, 2, 2, 2, 3, 4]


def _exponent(max_abs):
    """e with max|x| < 2^e (0 for an all-zero vector), from the bit pattern."""
    b = np.asarray(max_abs, dtype=np.float64).view(np.uint64)
    ex = (b >> np.uint64(52)).astype(np.int64)
    assert (ex[b != 0] > 0).all(), "normal inputs only in this test"
    return np.where(b == 0, 0, ex - 1022)


def _slices(x, e):
    """Five signed 8-bit slices of x relative to 2^e, along a new last axis."""
    b = x.view(np.uint64)
    ex = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (b & np.uint64((1 << 52) - 1)) | np.where(ex > 0, np.uint64(1 << 52), np.uint64(0))
    sh = 1075 - FB + e - np.maximum(ex, 1)
    assert (sh[x != 0] >= 13).all()
    F = np.where(sh >= 64, np.uint64(0), m >> np.minimum(sh, 63).astype(np.uint64))
    sign = np.where((b >> np.uint64(63)) != 0, -1, 1)
    return np.stack([sign * ((F >> np.uint64(FB - B * (s + 1))) & np.uint64(255)).astype(np.int64)
                     for s in range(NS)], axis=-1)


def _split_product(A, Y):
    """A (M x K) times Y (K x N) the way the kernel computes it."""
    K = A.shape[1]
    ea = _exponent(np.abs(A).max(axis=1))
    ey = _exponent(np.abs(Y).max(axis=0))
    qa = _slices(A, ea[:, None])            # M x K x NS
    qy = _slices(Y, ey[None, :])            # K x N x NS
    acc = np.zeros((8, A.shape[0], Y.shape[1]), dtype=np.float32)
    for k0 in range(0, K, 16):
        for s in range(NS):
            for t in range(NS - s):
                part = qa[:, k0:k0 + 16, s] @ qy[k0:k0 + 16, :, t]   # exact int64 (< 2^20)
                a = ACC[(s, t)]
                acc[a] = (acc[a] + part.astype(np.float32)).astype(np.float32)
                if DIAG[a] <= 2:
                    assert np.abs(acc[a]).max() < 2 ** 24
    total = np.zeros(acc.shape[1:], dtype=np.int64)
    for a in range(8):
        assert np.array_equal(acc[a], np.round(acc[a])), "accumulators hold integers"
        total += acc[a].astype(np.int64) << (B * (NS - 1 - DIAG[a]))
    pe = ea[:, None] + ey[None, :] - B * (NS + 1)
    return np.ldexp(total.astype(np.float64), pe)


def test_split_product_error_bound():
    rng = np.random.default_rng(11)
    M, K, N = 64, 256, 48
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-6, 6, (M, 1)))
    Y = rng.standard_normal((K, N)) * np.exp(rng.uniform(-6, 6, (1, N)))
    A[0] = np.abs(A[0])                     # same-sign row and column: no cancellation in the sums
    Y[:, 0] = np.abs(Y[:, 0])
    A[1] = 255.0 / 256.0 * 2.0 ** 3         # slices at their largest value
    Y[:, 1] = 255.0 / 256.0 * 2.0 ** -2
    P = _split_product(A, Y)
    ref = A @ Y
    bound = 2.0 ** -37 * K * np.abs(A).max(axis=1)[:, None] * np.abs(Y).max(axis=0)[None, :]
    assert (np.abs(P - ref) <= bound).all(), float((np.abs(P - ref) / bound).max())


def test_split_product_zero_rows_and_columns():
    rng = np.random.default_rng(12)
    A = rng.standard_normal((16, 256))
    Y = rng.standard_normal((256, 16))
    A[3] = 0.0
    Y[:, 5] = 0.0
    P = _split_product(A, Y)
    assert (P[3] == 0.0).all() and (P[:, 5] == 0.0).all()
