"""The dense unit columns' restructured recurrence, checked on the CPU.

unit_csc (src/sparseDist.cpp:246-284) walks a column's non-zeros once:
    if (scale < a) { r = scale / a; ssq = 1 + ssq * r * r; scale = a; }
    else           { r = a / scale; ssq += r * r; }
then u = (x / scale) / sqrt(ssq).  k_unit_dense (sparsedist_gb300/csrc/
sdg_exact.cu) computes the same values in another order of work: per 32-row
chunk, every ratio and branch from a prefix maximum of the magnitudes taken
on their IEEE bit patterns (integers order non-negative doubles), then each
column's chain over the chunk.  Both are restated here in Python (IEEE
doubles, no fused multiply-add); the sequential form is pinned to the
oracle's unit columns through its cosine similarity slab against one-hot
columns (sim(x_j, e_r) = u_j[r] exactly), and the chunked form must equal it
bit for bit, for every columns-per-warp split the kernel uses.
"""
import struct

import numpy as np
import scipy.sparse as sp

from backends import OracleBackend


def bits(v):
    return struct.unpack("<q", struct.pack("<d", v))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def unit_sequential(col):
    scale, ssq = 0.0, 1.0
    for v in col:
        if v == 0.0:
            continue
        a = abs(v)
        if scale < a:
            r = scale / a
            ssq = 1.0 + ssq * r * r
            scale = a
        else:
            r = a / scale
            ssq += r * r
    sq = np.sqrt(ssq)
    return np.array([0.0 if scale == 0.0 else (v / scale) / sq for v in col]), scale


def unit_chunked(X, cpw):
    """k_unit_dense's order of work for one d x n block (column-major)."""
    d, n = X.shape
    U = np.zeros_like(X)
    scales = np.zeros(n)
    for j0 in range(0, n, cpw):
        nc = min(cpw, n - j0)
        scale_bits = [0] * nc
        ssq = [1.0] * nc
        for k0 in range(0, d, 32):
            kn = min(32, d - k0)
            R = [[0.0] * nc for _ in range(kn)]
            F = [[0] * nc for _ in range(kn)]
            for c in range(nc):
                ab = [bits(X[k0 + l, j0 + c]) & 0x7FFFFFFFFFFFFFFF if l < kn else 0 for l in range(32)]
                incl, m = [], 0
                for l in range(32):
                    m = max(m, ab[l])
                    incl.append(m)
                for l in range(kn):
                    prev = max(incl[l - 1] if l else 0, scale_bits[c])
                    if ab[l] != 0:
                        av, pv = from_bits(ab[l]), from_bits(prev)
                        if prev < ab[l]:
                            F[l][c], R[l][c] = 1, pv / av
                        else:
                            F[l][c], R[l][c] = 2, av / pv
                scale_bits[c] = max(scale_bits[c], incl[31])
            for c in range(nc):
                for t in range(kn):
                    if F[t][c] == 1:
                        ssq[c] = 1.0 + ssq[c] * R[t][c] * R[t][c]
                    elif F[t][c] == 2:
                        ssq[c] = ssq[c] + R[t][c] * R[t][c]
        for c in range(nc):
            scale = from_bits(scale_bits[c])
            sq = np.sqrt(ssq[c])
            scales[j0 + c] = scale
            U[:, j0 + c] = [0.0 if scale == 0.0 else (v / scale) / sq for v in X[:, j0 + c]]
    return U, scales


def columns(rng, d):
    cols = [rng.standard_normal(d) * np.exp2(rng.integers(-40, 40, d)),
            np.where(rng.random(d) < 0.4, 0.0, rng.standard_normal(d)),
            np.arange(1, d + 1, dtype=np.float64) * 1.5,          # a new maximum at every row
            np.arange(d, 0, -1, dtype=np.float64) * 0.75,         # the maximum first
            np.full(d, -2.5),
            np.zeros(d),
            np.where(np.arange(d) == d - 1, 7.0, 0.0),            # one entry, in the last chunk
            np.where(np.arange(d) % 3 == 0, -0.0, 1e-300 * (1 + np.arange(d)))]
    for _ in range(5):
        cols.append(rng.standard_normal(d) * 10.0 ** rng.uniform(-150, 150))
    return np.stack(cols, axis=1)


def oracle_units(X):
    d, n = X.shape
    A = sp.csc_matrix(X)
    A.eliminate_zeros()
    E = sp.identity(d, format="csc")
    sim = OracleBackend().slab("cosine", A, E, dist=False)    # n x d: sim(x_j, e_r)
    return np.asarray(sim).T


def test_chunked_recurrence_equals_the_sequential_one_and_the_oracle():
    rng = np.random.default_rng(23)
    for d in (1, 31, 45, 64, 100):
        X = columns(rng, d)
        seq = np.stack([unit_sequential(X[:, j])[0] for j in range(X.shape[1])], axis=1)
        orc = oracle_units(X)
        nz = X != 0.0
        assert np.array_equal(seq[nz].view(np.uint64), orc[nz].view(np.uint64)), d
        for cpw in (8, 32):
            U, scales = unit_chunked(X, cpw)
            assert np.array_equal(U.view(np.uint64), seq.view(np.uint64)), (d, cpw)
            assert np.array_equal(scales, [unit_sequential(X[:, j])[1] for j in range(X.shape[1])])
