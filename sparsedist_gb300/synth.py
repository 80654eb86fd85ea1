"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark workloads (the reference's own bench reads 10x PBMC downloads,
bench/R/03-datasets.R:56-71, which are not available offline; these stand in
for them).

* ``uniform_csc``: nrow x ncol CSC, a uniform random pattern of exactly
  round(density * nrow * ncol) positions, |N(0,1)| values (the CPU-runnable
  case: 2,000 x 10,000 at 2%).
* ``logcount_csc``: single-cell-like log counts (the kNN-at-scale case:
  30,000 x 200,000): per-column nnz ~ lognormal(log(mean_nnz) - sdlog^2/2, sdlog)
  clipped to [1, nrow]; rows drawn without replacement with probability
  proportional to row means mu_r ~ lognormal(0, row_sdlog) (exponential-race
  sampling); values log1p(NB(size 2, mean mu_r * s_c)) with column scales
  s_c ~ lognormal(0, col_sdlog); zero counts are dropped, so no explicit zeros
  are stored.  Generated on the GPU with torch (seeded), returned as host
  numpy CSC arrays.
* ``cross_draw`` / ``cross_problem``: the batched uneven sparseKNNCross
  problems: per problem nq log-U[100, 50,000] query and nr log-U[1,000,
  200,000] reference columns, rows U[5,000, 30,000], density
  log-U[0.1 %, 10 %] (a uniform pattern: positions drawn uniformly and made
  unique), |N(0,1)| values; methods cycle binary / cosine / manhattan / js (js
  on column-normalised data), k drawn from {10, 20, 50}.
"""
from __future__ import annotations

import math

import numpy as np


def uniform_csc(nrow, ncol, density, seed=0):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    M = sp.random(nrow, ncol, density=density, format="csc", random_state=rng,
                  data_rvs=lambda n: np.abs(rng.standard_normal(n)))
    M.sort_indices()
    return M


def dense_embeddings(d=256, n=2000000, centres=1000, sigma=0.3, cluster_frac=0.5, dup_frac=0.01,
                     eps=1e-6, seed=0, device="cuda"):
    """The dense-embedding workload as a torch float32 tensor of shape (n, d)
    (i.e. d x n column-major): a share of i.i.d. N(0,1) columns, the rest drawn
    around one of ``centres`` N(0,1) centres with N(0, sigma^2) noise, then
    ``dup_frac`` of the columns replaced by a copy of another column plus
    N(0, eps^2) noise (near duplicates)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    X = torch.randn(n, d, generator=g, device=device, dtype=torch.float32)
    C = torch.randn(centres, d, generator=g, device=device, dtype=torch.float32)
    member = torch.rand(n, generator=g, device=device) < cluster_frac
    which = torch.randint(0, centres, (n,), generator=g, device=device)
    X = torch.where(member[:, None], C[which] + sigma * X, X)
    ndup = int(dup_frac * n)
    dst = torch.randperm(n, generator=g, device=device)[:ndup]
    src = torch.randint(0, n, (ndup,), generator=g, device=device)
    X[dst] = X[src] + eps * torch.randn(ndup, d, generator=g, device=device)
    return X.contiguous()


def logcount_csc(nrow=30000, ncol=200000, mean_nnz=1800.0, sdlog=0.6, row_sdlog=1.5,
                 col_sdlog=0.5, seed=0, device="cuda", chunk=1024, keep_on_device=False):
    """Returns (p int32[ncol+1], i int32[nnz], x float64[nnz]) on the host, or,
    with keep_on_device, as torch tensors on ``device`` (p included)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    f64 = torch.float64
    mu = torch.exp(torch.randn(nrow, generator=g, device=device, dtype=f64) * row_sdlog)
    meanlog = math.log(mean_nnz) - sdlog * sdlog / 2.0
    nnz_c = torch.exp(meanlog + sdlog * torch.randn(ncol, generator=g, device=device, dtype=f64))
    nnz_c = torch.clamp(torch.round(nnz_c), 1, nrow).to(torch.int64)
    s_c = torch.exp(col_sdlog * torch.randn(ncol, generator=g, device=device, dtype=f64))
    inv_mu = (1.0 / mu)[None, :]
    p = np.zeros(ncol + 1, np.int64)
    rows_parts, vals_parts = [], []
    for c0 in range(0, ncol, chunk):
        c1 = min(ncol, c0 + chunk)
        b = c1 - c0
        u = torch.rand(b, nrow, generator=g, device=device, dtype=f64)
        key = -torch.log1p(-u) * inv_mu                  # Exp(1) / mu_r: smallest keys win
        kth = torch.sort(key, dim=1).values.gather(1, (nnz_c[c0:c1] - 1)[:, None])
        mask = key <= kth
        cols, rows = mask.nonzero(as_tuple=True)         # column-major: col, then row ascending
        mean = mu[rows] * s_c[c0 + cols]
        lam = torch._standard_gamma(torch.full_like(mean, 2.0), generator=g) * (mean / 2.0)
        cnt = torch.poisson(lam, generator=g)
        keep = cnt > 0
        cols, rows, cnt = cols[keep], rows[keep], cnt[keep]
        vals = torch.log1p(cnt)
        per_col = torch.bincount(cols, minlength=b).cpu().numpy()
        p[c0 + 1:c1 + 1] = per_col
        if keep_on_device:
            rows_parts.append(rows.to(torch.int32))
            vals_parts.append(vals)
        else:
            rows_parts.append(rows.to(torch.int32).cpu().numpy())
            vals_parts.append(vals.cpu().numpy())
    p = np.cumsum(p)
    if p[-1] >= 2 ** 31:
        raise ValueError("nnz exceeds the dgCMatrix limit of 2^31 - 1")
    if keep_on_device:
        return (torch.from_numpy(p.astype(np.int32)).to(device), torch.cat(rows_parts),
                torch.cat(vals_parts))
    return p.astype(np.int32), np.concatenate(rows_parts), np.concatenate(vals_parts)


CROSS_METHODS = ("binary", "cosine", "manhattan", "js")


def cross_draw(n=512, seed=4, scale=1.0):
    """The parameters of the batched problems: a list of dicts (nq, nr, rows,
    density, method, k, seed); ``scale`` multiplies the column counts."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(n):
        nq = int(round(math.exp(rng.uniform(math.log(100), math.log(50000))) * scale))
        nr = int(round(math.exp(rng.uniform(math.log(1000), math.log(200000))) * scale))
        rows = int(rng.integers(5000, 30001))
        dens = math.exp(rng.uniform(math.log(0.001), math.log(0.1)))
        k = int(rng.choice([10, 20, 50]))
        out.append(dict(nq=max(1, nq), nr=max(1, nr), rows=rows, density=dens, method=CROSS_METHODS[p % 4], k=k,
                        seed=int(seed) * 100003 + p))
    return out


def _uniform_pattern(nrow, ncol, density, g, device):
    import torch
    m = int(round(density * nrow * ncol))
    keys = torch.unique(torch.randint(0, nrow * ncol, (max(m, 1),), generator=g, device=device))
    cols = keys // nrow
    rows = (keys - cols * nrow).to(torch.int32)
    vals = torch.randn(keys.numel(), generator=g, device=device, dtype=torch.float64).abs()
    counts = torch.bincount(cols, minlength=ncol)
    return counts, rows, vals, cols


def cross_problem(spec, device="cuda"):
    """(X, Y) of one batched problem as scipy CSC matrices (host)."""
    import scipy.sparse as sp
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(spec["seed"])
    mats = []
    for ncol in (spec["nq"], spec["nr"]):
        counts, rows, vals, cols = _uniform_pattern(spec["rows"], ncol, spec["density"], g, device)
        if spec["method"] == "js":
            sums = torch.zeros(ncol, dtype=torch.float64, device=device).index_add_(0, cols, vals)
            vals = vals / sums[cols]
        p = np.zeros(ncol + 1, np.int64)
        p[1:] = np.cumsum(counts.cpu().numpy())
        M = sp.csc_matrix((vals.cpu().numpy(), rows.cpu().numpy(), p.astype(np.int32)), shape=(spec["rows"], ncol))
        mats.append(M)
    return mats[0], mats[1]
