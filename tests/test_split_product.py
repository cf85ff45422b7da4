"""The arithmetic of the tensor-core FP64 panel products (panels_tc.cu, tc.cuh), restated in numpy.

Every row of a G block and every column of the right-hand-side block is written as eight signed
7-bit digits against a power-of-two scale (the truncated 56-bit fixed-point fraction of each value);
the product is the sum over digit pairs with p + q <= 9 of the integer products D_pq 2^(-7(p+q)),
grouped by the kernel into eight accumulators whose halves each sum at most four pair products.
Checked here: every accumulator half stays below 2^24 (so FP32 holds it exactly, as the tensor
cores accumulate it), and the result's error stays within the error bound of an FP64 dot product,
64 * 2^-53 * (|G| |V|), on blocks with rows and columns of very different magnitude."""
import numpy as np

DIGITS, BITS = 8, 7


def exp_bound(a):
    """Smallest e with |a| < 2^e (per element); a huge negative number for zeros."""
    m, e = np.frexp(np.abs(a))
    return np.where(a == 0, -2000, e)


def split(M, axis):
    """Digits of M along rows (axis=1) or columns (axis=0): (exponents, digits[p] as float)."""
    e = np.max(exp_bound(M), axis=axis, keepdims=True)
    y = np.abs(M) / np.ldexp(1.0, np.maximum(e, -1074))
    Y = np.floor(np.ldexp(y, 56)).astype(np.uint64)  # truncated 56-bit fraction
    digs = []
    for p in range(1, DIGITS + 1):
        d = ((Y >> np.uint64(56 - BITS * p)) & np.uint64(127)).astype(np.float64)
        digs.append(np.where(M < 0, -d, d))
    return e, digs


def split_product(G, V):
    eg, gd = split(G, 1)
    ev, vd = split(V, 0)
    out = np.zeros((G.shape[0], V.shape[1]))
    # accumulator k (top diagonal k = p + q, p odd): top half pairs (p, q), bottom half (p + 1, q)
    for k in range(9, 1, -1):
        top = np.zeros_like(out)
        bot = np.zeros_like(out)
        for p in range(1, 8, 2):
            q = k - p
            if 1 <= q <= DIGITS:
                top += gd[p - 1] @ vd[q - 1]
                bot += gd[p] @ vd[q - 1]
        assert np.all(np.abs(top) < 2 ** 24) and np.all(np.abs(bot) < 2 ** 24)
        out += np.ldexp(top, -BITS * k) + np.ldexp(bot, -BITS * (k + 1))
    return out * np.ldexp(1.0, np.where(eg == -2000, 0, eg)) * np.ldexp(1.0, np.where(ev == -2000, 0, ev))


def test_split_product_reaches_fp64_dot_product_accuracy():
    rng = np.random.default_rng(0)
    for trial in range(8):
        G = rng.uniform(-1, 1, (64, 64)) * np.ldexp(1.0, rng.integers(-40, 40, (64, 1)))
        G[rng.random((64, 64)) < 0.25] *= 1e-12
        G[rng.random((64, 64)) < 0.1] = 0.0
        V = rng.uniform(-1, 1, (64, 16)) * np.ldexp(1.0, rng.integers(-30, 30, (1, 16)))
        ref = G @ V
        got = split_product(G, V)
        bound = 64 * 2.0 ** -53 * (np.abs(G) @ np.abs(V))
        assert np.all(np.abs(got - ref) <= bound), trial


def test_split_product_zero_rows_and_columns():
    G = np.zeros((64, 32))
    G[3, :] = np.linspace(-1, 1, 32)
    V = np.zeros((32, 16))
    V[:, 2] = 1.0
    got = split_product(G, V)
    assert np.array_equal(got[:, [0, 1] + list(range(3, 16))], np.zeros((64, 15)))
    assert abs(got[3, 2] - np.sum(G[3, :])) <= 1e-15
