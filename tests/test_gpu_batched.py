"""Batched uneven problems (the shape of the 512-problem batch, at test size): many
independent sparseKNNCross problems whose sizes are drawn log-uniformly,
with the methods cycling binary / cosine / manhattan / js (js on
column-normalised data) and k cycling 10 / 20 / 50, as in the full batch
(512 problems, nq log-U[100, 50,000], nr log-U[1,000, 200,000], rows
U[5,000, 30,000], density log-U[0.1 %, 10 %]).  Here nq, nr and the rows
are scaled down so that the oracle finishes in seconds.

Each problem's forward and reverse results must equal the oracle's
(bit for bit for the pinned methods; js within 1e-12 relative with a
tie-aware idx check), both run one after another and with every problem in
flight at once on four host threads, each owning one context and stream
(the library's work from different problems interleaving on the device)."""
import concurrent.futures as cf
import math

import numpy as np
import pytest

from backends import GpuBackend, OracleBackend, make_x, normalise_cols
from parity_cases import _knn_equal

pytestmark = pytest.mark.gpu

METHODS = ["binary", "cosine", "manhattan", "js"]
KS = [10, 20, 50]


def log_uniform(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def problems(n=24, seed=404):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(n):
        nq = log_uniform(rng, 20, 600)
        nr = log_uniform(rng, 100, 3000)
        rows = int(rng.integers(500, 3001))
        dens = math.exp(rng.uniform(math.log(0.001), math.log(0.10)))
        method, k = METHODS[t % 4], KS[t % 3]
        X = make_x(rows, nq, dens, 10000 + 2 * t)
        Y = make_x(rows, nr, dens, 10001 + 2 * t)
        if method == "js":
            X, Y = normalise_cols(X), normalise_cols(Y)
            if X.shape[1] == 0 or Y.shape[1] == 0:
                continue
        out.append(dict(X=X, Y=Y, method=method, k=k, tag="%d:%s nq=%d nr=%d rows=%d dens=%.4f k=%d"
                        % (t, method, X.shape[1], Y.shape[1], rows, dens, k)))
    return out


PROBLEMS = problems()


@pytest.fixture(scope="module")
def wanted():
    orc = OracleBackend()
    return [orc.knn_cross(p["X"], p["Y"], k=p["k"], method=p["method"]) for p in PROBLEMS]


def check(p, got, want):
    (fi, fd), (ri, rd), fl = got
    (wfi, wfd), (wri, wrd), wfl = want
    assert fl == wfl, p["tag"]
    assert _knn_equal(p["method"], True, (fi, fd), (wfi, wfd)), p["tag"] + " forward"
    assert _knn_equal(p["method"], True, (ri, rd), (wri, wrd)), p["tag"] + " reverse"


@pytest.mark.parametrize("engine", [0, 2], ids=["auto", "screen"])
def test_batched_uneven_cross_problems_one_by_one(gpu, wanted, engine):
    gpu.set_engine(engine)
    try:
        for p, want in zip(PROBLEMS, wanted):
            got = gpu.knn_cross(p["X"], p["Y"], k=p["k"], method=p["method"])
            check(p, got, want)
    finally:
        gpu.set_engine(0)


def test_batched_uneven_cross_problems_all_in_flight(wanted):
    # a context belongs to one thread at a time: thread s owns context s and
    # runs problems s, s + 4, s + 8, ...
    backends = [GpuBackend() for _ in range(4)]

    def run_shard(sh):
        out = []
        for t in range(sh, len(PROBLEMS), 4):
            p = PROBLEMS[t]
            out.append((t, backends[sh].knn_cross(p["X"], p["Y"], k=p["k"], method=p["method"])))
        return out

    with cf.ThreadPoolExecutor(4) as ex:
        shards = list(ex.map(run_shard, range(4)))
    got = dict(item for shard in shards for item in shard)
    assert sorted(got) == list(range(len(PROBLEMS)))
    for t, (p, want) in enumerate(zip(PROBLEMS, wanted)):
        check(p, got[t], want)


def _batch(problems, ctx=None):
    from backends import METHODS as CODES
    from sparsedist_gb300 import _lib
    ctx = ctx or _lib.Context()
    return _lib.knn_cross_batch(ctx, [(p["X"], p["Y"], CODES[p["method"]], True, p["k"]) for p in problems])


def test_batch_call_equals_oracle_twice(wanted):
    """Every problem in ONE sdg_knn_cross_batch call (the exact-path searches
    of the call in one persistent launch, the others on the screened engines
    the autotuner picks), twice in a row on one context: the autotuner has
    learned from the first call's timings and may pick other engines in the
    second, whose results must still equal the oracle's."""
    from sparsedist_gb300 import _lib
    ctx = _lib.Context()
    for rnd in range(2):
        rc, res = _batch(PROBLEMS, ctx)
        assert rc == 0
        for p, r, want in zip(PROBLEMS, res, wanted):
            assert r["status"] == 0, p["tag"]
            assert all(e in (1, 2, 3) for e in r["engines"]), p["tag"]
            check(p, (r["forward"], r["reverse"], r["flags"]), want)
    used = {e for r in res for e in r["engines"]}
    assert 1 in used                               # the persistent exact launch ran


def test_batch_call_keeps_each_problems_status():
    """A problem that fails validation (row dimensions differ) or has no
    candidate (every reference column empty) reports its own status and
    message; the problems around it are computed as usual, and clamped k
    sets the warning flags as sparseKNNCross's clamp does."""
    import scipy.sparse as sp
    from sparsedist_gb300 import _lib
    good = PROBLEMS[:3]
    X = make_x(300, 40, 0.05, 7)
    bad_rows = dict(X=X, Y=make_x(301, 30, 0.05, 8), method="cosine", k=5, tag="rows")
    empty = dict(X=X, Y=sp.csc_matrix((300, 12)), method="binary", k=5, tag="no candidates")
    clamp = dict(X=make_x(300, 6, 0.2, 9), Y=make_x(300, 4, 0.2, 10), method="cosine", k=10, tag="clamp")
    probs = good + [bad_rows, empty, clamp]
    rc, res = _batch(probs)
    assert rc == -3                                # the first failure: SDG_E_ROWS
    assert [r["status"] for r in res[3:5]] == [-3, -4]
    orc = OracleBackend()
    for p, r in zip(good + [clamp], res[:3] + res[5:]):
        want = orc.knn_cross(p["X"], p["Y"], k=p["k"], method=p["method"])
        check(p, (r["forward"], r["reverse"], r["flags"]), want)
    assert res[5]["flags"] == 3 and res[5]["forward"][0].shape == (6, 4) and res[5]["reverse"][0].shape == (4, 6)
