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


# ---- js: the FP32 screen of fastJS2 (sparsedist_gb300/csrc/sdg_screen.cu,
# accumulate_js and js_key_and_bound).  Per shared row the kernel computes
# g = ((S log S) - xlogx(P)) - xlogx(Q) with p, q the FP32 values, S = p + q,
# the __logf intrinsic (taken within 2^-20.41 absolute on [0.5, 2], 6 ulp
# elsewhere: twice its documented accuracy, checked on the GPU),
# the stored FP32 x log x values and every operation rounded once, and sums the
# rows in FP32.  Here the logarithm is emulated at the edges of that error
# (the FP64 logarithm moved by up to the documented error, then rounded to
# FP32), rows are summed in random orders, and |G~ - G| must stay within
# u (33.5 (A_P + A_Q) + 0.75 n (C_P + C_Q)) 1.01, A = a column's sum of
# |x log x| + x, C = its sum.

def _f32(x):
    return np.float32(x)


def _logf_1ulp(S, rng):
    """The logarithm as __logf may return it: the FP64 logarithm moved by up to
    the error the screen allows (2^-20.41 absolute on [0.5, 2]; 6 ulp of the
    result elsewhere), towards either side, rounded to FP32."""
    t = np.log(np.float64(S))
    if 0.5 <= float(S) <= 2.0:
        e = 2.0 ** -20.41
    else:
        e = 6.0 * float(np.spacing(np.float32(abs(t))))
    return np.float32(t + e * rng.choice([-1.0, 1.0]) * rng.uniform(0.9, 1.0))


def _js_case(P, Q, rng):
    """P, Q: the two columns' values (dense vectors, 0 = not stored)."""
    shared = (P != 0) & (Q != 0)
    def xlx(v):
        with np.errstate(divide="ignore", invalid="ignore"):
            r = v * np.log(v)
        return np.where(v > 0, r, 0.0)
    def A(v):
        return float(np.float32(np.sum(np.abs(xlx(v)) + v) * (1 + 1e-12)))   # ~rounded up
    AP, AQ = A(P), A(Q)
    n = int(min(np.count_nonzero(P), np.count_nonzero(Q)))
    idx = np.flatnonzero(shared)
    # exact G without cancellation: g = P log1p(Q/P) + Q log1p(P/Q)
    Ps, Qs = P[idx], Q[idx]
    G = float(np.sum(Ps * np.log1p(Qs / Ps) + Qs * np.log1p(Ps / Qs)))
    terms = []
    for a, b in zip(Ps, Qs):
        p, q = _f32(a), _f32(b)
        xp, xq = _f32(a * np.log(a)), _f32(b * np.log(b))
        S = _f32(p + q)
        t1 = _f32(S * _logf_1ulp(S, rng))
        terms.append(_f32(_f32(t1 - xp) - xq))
    CP, CQ = float(P.sum()), float(Q.sum())
    bound = 2.0 ** -24 * (33.5 * (AP + AQ) + 0.75 * n * (CP + CQ)) * 1.01
    worst = 0.0
    for _ in range(3):
        acc = np.float32(0)
        for t in np.asarray(terms, np.float32)[rng.permutation(len(terms))]:
            acc = _f32(acc + t)
        err = abs(float(acc) - G)
        assert err <= bound, (err, bound, n)
        worst = max(worst, err / bound if bound > 0 else 0.0)
    return worst


def _js_pair(rng, nrow, density, draw):
    P = np.zeros(nrow)
    Q = np.zeros(nrow)
    ip = rng.random(nrow) < density
    iq = rng.random(nrow) < density
    P[ip] = draw(rng, ip.sum())
    Q[iq] = draw(rng, iq.sum())
    return P, Q


def test_js_bound_normalised_columns():
    rng = np.random.default_rng(21)
    for _ in range(25):
        P, Q = _js_pair(rng, 3000, 0.2, lambda g, m: g.random(m) + 1e-3)
        P /= P.sum()
        Q /= Q.sum()
        assert _js_case(P, Q, rng) < 1.0


def test_js_bound_skewed_ratios_and_ranges():
    rng = np.random.default_rng(22)
    # values over [2^-90, 2^90] in log scale, so that shared rows pair tiny
    # with huge values (Q << P), plus exact ties P == Q
    for _ in range(20):
        P, Q = _js_pair(rng, 2000, 0.3, lambda g, m: np.exp2(g.uniform(-90, 90, m)))
        tie = (P != 0) & (Q != 0) & (rng.random(2000) < 0.2)
        Q[tie] = P[tie]
        assert _js_case(P, Q, rng) < 1.0


def test_js_bound_counts_above_one():
    rng = np.random.default_rng(23)
    for _ in range(20):
        P, Q = _js_pair(rng, 4000, 0.1, lambda g, m: g.negative_binomial(2, 0.1, m).astype(float) + 1.0)
        assert _js_case(P, Q, rng) < 1.0


# ---- pearson / covariance: the FP32 product screen with the moment key
# (sparsedist_gb300/csrc/sdg_screen.cu, moment_key_and_bound).  The screen's
# s~ is the FP32 FMA chain over the matched rows' FP32 values (emulated here as
# the FP64 product-plus-sum rounded once to FP32); the interval [key - err,
# key + err] must contain the exact path's value (pearson_finish /
# covariance_finish: FP64 sums in row order, then the clamp and the
# non-finite-to-0 rule) for signed values, tiny and near-constant columns.

U = 2.0 ** -24


def _moment_bounds(pearson, s, n, N, SP, SSP, SQ, SSQ):
    norm = N - 1.0 if N > 1 else 1.0
    Es = ((n + 4.0) * U * 1.01) * np.sqrt(SSP * SSQ) + 1e-300
    m = (SP * SQ) / N
    cov = (s - m) / norm
    Ecov = (Es + 2.0 ** -50 * (abs(s) + abs(m))) / norm
    if not pearson:
        lo, hi = cov - Ecov * 1.0001, cov + Ecov * 1.0001
    else:
        vp = (SSP - (SP * SP) / N) / norm
        vq = (SSQ - (SQ * SQ) / N) / norm
        with np.errstate(invalid="ignore"):
            den = np.sqrt(vp) * np.sqrt(vq)
        if not (den > 0.0) or not np.isfinite(den):
            return 0.0, 0.0
        if den < 1e-200:
            return 0.0, 1.0001
        c = cov / den
        e = (Ecov / den + 2.0 ** -50 * abs(c)) * 1.0001
        lo, hi = min(1.0, max(-1.0, c - e)), min(1.0, max(-1.0, c + e))
    key = np.float32(0.5 * (lo + hi))
    err = np.float32(0.5 * (hi - lo)) + np.float32(2 * U * (abs(float(key)) + 1.0)) + np.float32(1e-30)
    return float(key), float(err)


def _exact_value(pearson, A, B):
    N = float(len(A))
    norm = N - 1.0 if N > 1 else 1.0
    sab = 0.0
    for a, b in zip(A, B):
        if a != 0 and b != 0:
            sab = sab + a * b
    cov = (sab - (A.sum() * B.sum()) / N) / norm
    if not pearson:
        return cov
    va = (np.dot(A, A) - (A.sum() * A.sum()) / N) / norm
    vb = (np.dot(B, B) - (B.sum() * B.sum()) / N) / norm
    with np.errstate(invalid="ignore", divide="ignore"):
        c = cov / (np.sqrt(va) * np.sqrt(vb))
    if not np.isfinite(c):
        c = 0.0
    return min(1.0, max(-1.0, c))


def _moment_case(A, B, rng):
    shared = np.flatnonzero((A != 0) & (B != 0))
    n = int(min(np.count_nonzero(A), np.count_nonzero(B)))
    acc = np.float32(0)
    for i in shared:                                        # the reference column's row order
        acc = np.float32(float(np.float32(A[i])) * float(np.float32(B[i])) + float(acc))
    for pearson in (True, False):
        key, err = _moment_bounds(pearson, float(acc), n, float(len(A)), float(A.sum()), float(np.dot(A, A)),
                                  float(B.sum()), float(np.dot(B, B)))
        v = _exact_value(pearson, A, B)
        assert key - err <= v <= key + err, (pearson, key, err, v)


def test_moment_bounds_cover_signed_and_degenerate_columns():
    rng = np.random.default_rng(31)
    for trial in range(60):
        nrow = int(rng.integers(50, 3000))
        dens = float(rng.uniform(0.02, 0.6))
        A = np.where(rng.random(nrow) < dens, rng.standard_normal(nrow) * 10 ** rng.uniform(-3, 3), 0.0)
        B = np.where(rng.random(nrow) < dens, rng.standard_normal(nrow) * 10 ** rng.uniform(-3, 3), 0.0)
        if trial % 5 == 0:
            B = A * 3.0 + (A != 0) * 1e-9              # nearly collinear: c close to 1
        if trial % 7 == 0:
            A[:] = 0.0
            A[:nrow // 2] = 2.5                        # near-constant pattern
        if trial % 11 == 0:
            B[:] = 1.25                                # constant column: zero variance, value 0
        _moment_case(A, B, rng)


# ---- the dense screen's per-pair bound (sparsedist_gb300/csrc/sdg_dense_tc.cu,
# tight_bounds): BF16 copies (FP64 -> FP32 -> BF16, round to nearest even as
# __float2bfloat16_rn), exact BF16 products in FP32, FP32 sums in random
# orders; |sum b_q b_r - sum v_q v_r| <= (e_q ||v_r|| + ||b_q|| e_r + (d + 64)
# 2^-21 ||b_q|| ||b_r||) 1.01 for unit columns (cosine) and raw columns
# (euclidean's inner product).

def _bf16(x):
    f = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (f >> 16) & 1
    r = ((f + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _dense_case(vq, vr, rng, unit):
    bq, br = _bf16(vq), _bf16(vr)
    eq, er = np.linalg.norm(vq - bq) * (1 + 1e-12), np.linalg.norm(vr - br) * (1 + 1e-12)
    nq, nr = np.linalg.norm(bq) * (1 + 1e-12), np.linalg.norm(br) * (1 + 1e-12)
    d = len(vq)
    vnorm = 1.000001 if unit else float(np.linalg.norm(vr)) * 1.000001
    bound = (eq * vnorm + nq * er + (d + 64) * 2.0 ** -21 * nq * nr) * 1.01 + 1e-12
    exact = float(np.dot(vq, vr))
    prods = (bq * br).astype(np.float32)
    assert np.all(prods.astype(np.float64) == bq * br)          # exact in FP32
    worst = 0.0
    for _ in range(3):
        acc = np.float32(0)
        for t in prods[rng.permutation(d)]:
            acc = np.float32(acc + t)
        err = abs(float(acc) - exact)
        assert err <= bound, (err, bound)
        worst = max(worst, err / bound)
    return worst


def test_dense_bf16_pair_bound():
    rng = np.random.default_rng(41)
    worst = 0.0
    for trial in range(40):
        d = int(rng.choice([32, 64, 96, 256]))
        vq, vr = rng.standard_normal(d), rng.standard_normal(d)
        if trial % 3 == 0:
            vr = vq + 1e-6 * rng.standard_normal(d)                # near duplicate
        unit = trial % 2 == 0
        if unit:
            vq, vr = vq / np.linalg.norm(vq), vr / np.linalg.norm(vr)
        worst = max(worst, _dense_case(vq, vr, rng, unit))
    assert worst < 1.0


# The dense path's third cut (sdg_dense.cu, k_dense_refine_dot): a warp
# accumulates lane l's share of the FP32 copies with FMA (the float4s l,
# l + 32, ... when d is a multiple of 4, else the elements l, l + 32, ...), a
# five-level xor butterfly adds the lanes, and the result must lie
# within C Nq Nr + 1e-15 (cosine; N = ||bf16 copy|| + ||copy error|| rounded
# up) or C m + 1e-36 (euclidean, m the FP32 sum of squares) of the FP64 value
# the exact stage computes (sequential, unfused, ascending rows).

def _gam(m, u):
    return m * u / (1.0 - m * u)


def _lane_elements(d):
    """Each lane's elements in the kernel's order, and J (the longest chain)."""
    if d % 4 == 0:
        lanes = [[4 * f + c for f in range(lane, d // 4, 32) for c in range(4)] for lane in range(32)]
        J = 4 * ((d + 127) // 128)
    else:
        lanes = [list(range(lane, d, 32)) for lane in range(32)]
        J = (d + 31) // 32
    assert max(len(e) for e in lanes) <= J and sorted(sum(lanes, [])) == list(range(d))
    return lanes, J


def _refine_constant(cosine, d):
    u, u53, J = 2.0 ** -24, 2.0 ** -53, _lane_elements(d)[1]
    if cosine:
        c = _gam(J + 5, u) * (1 + u) ** 2 + 2 * u + u * u + _gam(d + 1, u53)
    else:
        c = (_gam(J + 7, u) + _gam(d + 2, u53)) / (1 - _gam(J + 7, u))
    return ru32(c * 1.01 * (1 + 1e-12))


def _fma32(a, b, c):
    # a * b is exact in FP64 for FP32 a, b; one more FP64 rounding before the
    # FP32 one (at most 2^-29 of an FP32 ulp beyond a single rounding)
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def _warp_dot(a32, b32, square_diff):
    d = len(a32)
    lanes = np.zeros(32, np.float32)
    for lane, elems in enumerate(_lane_elements(d)[0]):
        acc = np.float32(0)
        for e in elems:
            if square_diff:
                df = np.float32(a32[e] - b32[e])
                acc = _fma32(df, df, acc)
            else:
                acc = _fma32(a32[e], b32[e], acc)
        lanes[lane] = acc
    for o in (16, 8, 4, 2, 1):
        lanes = (lanes + lanes[np.arange(32) ^ o]).astype(np.float32)
    assert np.all(lanes == lanes[0])               # the butterfly leaves one value on every lane
    return float(lanes[0])


def _seq64(a, b, square_diff):
    acc = 0.0
    for x, y in zip(a, b):
        if square_diff:
            t = x - y
            acc = acc + t * t
        else:
            acc = acc + x * y
    return acc


def _refine_cosine_case(vq, vr):
    uq, ur = vq / np.linalg.norm(vq), vr / np.linalg.norm(vr)
    Ns = []
    for u in (uq, ur):
        b = _bf16(u)
        Ns.append(ru32(ru32(np.linalg.norm(b) * (1 + 1e-12)) + ru32(np.linalg.norm(u - b) * (1 + 1e-12))))
    s = _warp_dot(ur.astype(np.float32), uq.astype(np.float32), False)
    c = _seq64(ur, uq, False)
    bound = _refine_constant(True, len(vq)) * Ns[0] * Ns[1] + 1e-15
    assert abs(s - c) <= bound, (abs(s - c), bound)
    return abs(s - c) / bound


def _refine_euclid_case(xq, xr):
    xq, xr = xq.astype(np.float32), xr.astype(np.float32)
    m = _warp_dot(xr, xq, True)
    num = _seq64(xr.astype(np.float64), xq.astype(np.float64), True)
    bound = _refine_constant(False, len(xq)) * m + 1e-36
    assert abs(m - num) <= bound, (abs(m - num), bound)
    return abs(m - num) / bound


def test_dense_fp32_cut_bound():
    rng = np.random.default_rng(73)
    worst = 0.0
    for trial in range(60):
        d = int(rng.choice([1, 5, 31, 33, 64, 100, 132, 256, 260]))
        kind = trial % 5
        vq = rng.standard_normal(d)
        if kind == 0:
            vr = rng.standard_normal(d)
        elif kind == 1:
            vr = vq + 1e-7 * rng.standard_normal(d)                # near duplicate
        elif kind == 2:
            vr = vq.copy()                                         # duplicate
        elif kind == 3:
            vq = np.abs(vq) + 1.0                                  # every product positive and alike:
            vr = np.full(d, 1.0) + 1e-3 * rng.standard_normal(d)   # the roundings pile up one way
        else:
            vq = vq * np.exp2(rng.integers(-30, 30, d))            # wide exponent range
            vr = vq * (1 + 1e-4 * rng.standard_normal(d))
        worst = max(worst, _refine_cosine_case(vq, vr))
        worst = max(worst, _refine_euclid_case(vq * 3.0, vr * 3.0))
    assert worst < 1.0


def _rd32(x):
    """An FP32 value at or below the real x (round to nearest, then one step
    down when that went up): the kernel's __fsub_rd / __fadd_rd stand-in."""
    f = np.float32(x)
    return f if float(f) <= x else np.nextafter(f, np.float32(-np.inf))


def _ru32(x):
    f = np.float32(x)
    return f if float(f) >= x else np.nextafter(f, np.float32(np.inf))


def _dense_cut32(T):
    T = np.float32(T)
    return np.float32(T - np.float32(np.float32(abs(T)) * np.float32(2.0 ** -21) + np.float32(1e-30)))


def test_dense_fp32_cut_keeps_the_exact_top_k_with_near_ties():
    """k_dense_refine_cut's selection on candidates the FP32 products cannot
    separate: 150 references at relative offsets 2^-25 .. 2^-12 from the
    query and 4 exact copies (distance ties broken by index); T3 = the k-th
    largest lower bound, every candidate with hi >= dense_cut(T3) kept.  Every
    reference whose FP64 distance is at most the k-th smallest must be kept."""
    rng = np.random.default_rng(31)
    d, k = 256, 20
    C = _refine_constant(True, d)
    for trial in range(3):
        q = rng.standard_normal(d)
        R = [q * (1 + s * rng.standard_normal(d)) for s in np.exp2(rng.uniform(-25, -12, 150))]
        R += [q.copy() for _ in range(4)]
        R += [rng.standard_normal(d) for _ in range(30)]
        R = np.asarray(R, np.float32).astype(np.float64)          # FP32 inputs, as the dense path takes
        q = q.astype(np.float32).astype(np.float64)
        uq = q / np.linalg.norm(q)
        U = R / np.linalg.norm(R, axis=1)[:, None]
        bq = _bf16(uq)
        Nq = ru32(ru32(np.linalg.norm(bq) * (1 + 1e-12)) + ru32(np.linalg.norm(uq - bq) * (1 + 1e-12)))
        lo, hi, dist = [], [], []
        for ur in U:
            c = _seq64(ur, uq, False)
            dist.append(1.0 - min(1.0, max(-1.0, c)))
            s = _warp_dot(ur.astype(np.float32), uq.astype(np.float32), False)
            br = _bf16(ur)
            Nr = ru32(ru32(np.linalg.norm(br) * (1 + 1e-12)) + ru32(np.linalg.norm(ur - br) * (1 + 1e-12)))
            E = float(_ru32(C * float(_ru32(Nq * Nr)) + 1e-15))
            lo.append(_rd32(s - E))
            hi.append(_ru32(s + E))
        lo, hi, dist = np.array(lo), np.array(hi), np.array(dist)
        cut = _dense_cut32(np.sort(lo)[::-1][k - 1])
        kept = hi >= cut
        kth = np.sort(dist)[k - 1]
        assert np.all(kept[dist <= kth]), trial
        assert k <= kept.sum() < len(kept)                          # the unrelated references go


def test_dense_fp32_cut_keeps_the_exact_top_k_euclidean():
    """The same selection for euclidean: key -m with m the FP32 sum of squared
    FP32 differences of the inputs, allowance C m + 1e-36; references at
    relative offsets 2^-24 .. 2^-10 from the query, exact copies (distance 0,
    ties) and unrelated references."""
    rng = np.random.default_rng(37)
    d, k = 256, 20
    C = _refine_constant(False, d)
    for trial in range(3):
        q = (rng.standard_normal(d) * 3.0).astype(np.float32)
        R = [q * (1 + s * rng.standard_normal(d)) for s in np.exp2(rng.uniform(-24, -10, 150))]
        R += [q.copy() for _ in range(3)]
        R += [rng.standard_normal(d) * 3.0 for _ in range(30)]
        R = np.asarray(R, np.float32)
        lo, hi, dist = [], [], []
        for r in R:
            num = _seq64(r.astype(np.float64), q.astype(np.float64), True)
            dist.append(np.sqrt(num))
            m = _warp_dot(r, q, True)
            E = float(_ru32(C * m + 1e-36))
            lo.append(_rd32(-m - E))
            hi.append(_ru32(-m + E))
        lo, hi, dist = np.array(lo), np.array(hi), np.array(dist)
        cut = _dense_cut32(np.sort(lo)[::-1][k - 1])
        kept = hi >= cut
        kth = np.sort(dist)[k - 1]
        assert np.all(kept[dist <= kth]), trial
        assert k <= kept.sum() < len(kept)
