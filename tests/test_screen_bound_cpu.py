"""The tensor-core screen's error bound, checked on the CPU.

The screen multiplies FP16 copies of the screen values (values below FP16's
smallest normal stored as 0) with FP32 accumulation, and bounds the
difference from the exact inner product by

    E = (1.000001 eq ||v_r|| + bq er + (n + 64) 2^-21 bq br) * 1.01 (+ tiny)

with eq, er the copies' exact rounding-error norms, bq, br the copies' norms
and n = min(nnz_q, nnz_r) (sparsedist_gb300/csrc/sdg_screen.cu, tc_bounds).
Here the copies are made with numpy's IEEE float16 rounding, the products
are summed in FP32 in arbitrary orders (the tensor cores' order is not
specified), and the bound must cover the difference every time — for unit
columns (cosine), raw values (euclidean's inner product) and 0 / 1 patterns
(binary), including values that fall below FP16's normal range.
"""
import numpy as np

HALF_MIN_NORMAL = 2.0 ** -14
ACC_ULP = 2.0 ** -21


def fp16_copy(v):
    f = v.astype(np.float32)
    f = np.where(np.abs(f) < HALF_MIN_NORMAL, np.float32(0), f)
    return f.astype(np.float16).astype(np.float64)


def ru32(x):
    """x rounded up to FP32 (the device stores the norms that way)."""
    f = np.float32(x)
    return float(f) if float(f) >= x else float(np.nextafter(f, np.float32(np.inf)))


def fp32_sum(terms, rng):
    order = rng.permutation(len(terms))
    acc = np.float32(0)
    for t in terms[order]:
        acc = np.float32(acc + np.float32(t))
    return float(acc)


def check_pairs(make_pair, unit, trials, seed):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for _ in range(trials):
        vq, vr = make_pair(rng)
        if unit:
            vq = vq / np.linalg.norm(vq) if np.any(vq) else vq
            vr = vr / np.linalg.norm(vr) if np.any(vr) else vr
        bq, br = fp16_copy(vq), fp16_copy(vr)
        eq, er = ru32(np.linalg.norm(vq - bq) * (1 + 1e-12)), ru32(np.linalg.norm(vr - br) * (1 + 1e-12))
        nq, nr = ru32(np.linalg.norm(bq) * (1 + 1e-12)), ru32(np.linalg.norm(br) * (1 + 1e-12))
        n = min(np.count_nonzero(vq), np.count_nonzero(vr))
        vnorm = 1.0 if unit else float(np.linalg.norm(vr))
        bound = (1.000001 * eq * vnorm + nq * er + (n + 64) * ACC_ULP * nq * nr) * 1.01 + 1e-12
        exact = float(np.dot(vq, vr))
        prods = bq * br                          # exact in FP32 (11-bit significands)
        assert np.all(prods.astype(np.float32).astype(np.float64) == prods)
        for _ in range(3):
            got = fp32_sum(prods[prods != 0], rng)
            err = abs(got - exact)
            assert err <= bound, (err, bound)
            worst = max(worst, err / bound)
    return worst


def _sparse_pair(rng, nrow, density, scale_fn):
    q = np.zeros(nrow)
    r = np.zeros(nrow)
    iq = rng.random(nrow) < density
    ir = rng.random(nrow) < density
    q[iq] = scale_fn(rng, iq.sum())
    r[ir] = scale_fn(rng, ir.sum())
    return q, r


def test_bound_covers_unit_columns():
    worst = check_pairs(lambda rng: _sparse_pair(rng, 3000, 0.3, lambda g, m: np.abs(g.standard_normal(m))),
                        unit=True, trials=40, seed=1)
    assert worst < 1.0


def test_bound_covers_tiny_and_wide_ranges():
    # unit values spanning 2^-20 .. 1: the smallest ones are stored as 0 and
    # their whole magnitude is in the rounding-error norm
    def wide(g, m):
        return np.exp(g.uniform(np.log(2.0 ** -20), 0.0, m))
    worst = check_pairs(lambda rng: _sparse_pair(rng, 4000, 0.2, wide), unit=True, trials=30, seed=2)
    assert worst < 1.0


def test_bound_covers_raw_values_and_patterns():
    def logcounts(g, m):
        return np.log1p(g.negative_binomial(2, 0.2, m).astype(float) + 1.0)
    check_pairs(lambda rng: _sparse_pair(rng, 5000, 0.1, logcounts), unit=False, trials=30, seed=3)
    check_pairs(lambda rng: _sparse_pair(rng, 5000, 0.1, lambda g, m: np.ones(m)), unit=False, trials=30,
                seed=4)
