"""Seeded synthetic matrices and start vectors for the IRLM workloads.

Every random number comes from SplitMix64 (Steele, Lea & Flood, "Fast
splittable pseudorandom number generators", OOPSLA 2014) used as a
counter-based generator:

    key(seed, stream) = mix(seed * 0xD1B54A32D192ED03 + stream)
    u64(seed, stream, i) = mix(key + (i + 1) * 0x9E3779B97F4A7C15)
    uniform01 = (u64 >> 11) * 2**-53                      in [0, 1)

(all arithmetic modulo 2**64; ``mix`` is the SplitMix64 output function).
Normal deviates use the Box-Muller transform (Box & Muller 1958).  The C++
library draws the default start vector of ``ds_solver_gpu`` with the same
formula (stream 0), so numpy and the library produce bit-identical vectors.

Matrices are returned as general (both triangles stored) CSR with int32
indices, columns ascending within each row, as a ``CSR`` tuple.
"""
from __future__ import annotations

from typing import NamedTuple

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_KEYMUL = np.uint64(0xD1B54A32D192ED03)

STREAM_START = 0       # start vector of the Lanczos process
STREAM_SHIFT = 1       # diagonal shift of the 3-D Laplacian
STREAM_GRAPH = 2       # Chung-Lu endpoint draws
STREAM_BAND = 3        # banded random matrix entries


class CSR(NamedTuple):
    n: int
    ncols: int
    row_ptr: np.ndarray   # int32 [n+1]
    col: np.ndarray       # int32 [nnz]
    val: np.ndarray       # float64 [nnz]

    @property
    def nnz(self) -> int:
        return int(self.col.shape[0])


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        z = np.array([np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * _KEYMUL + np.uint64(stream)],
                     dtype=np.uint64)
    return _mix(z)[0]


def u64(seed: int, stream: int, count: int, offset: int = 0) -> np.ndarray:
    """count raw 64-bit draws of (seed, stream) starting at index offset."""
    i = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(_key(seed, stream) + i * _GAMMA)


def uniform01(seed: int, stream: int, count: int, offset: int = 0) -> np.ndarray:
    return (u64(seed, stream, count, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform_pm1(seed: int, stream: int, count: int, offset: int = 0) -> np.ndarray:
    """Uniform on [-1, 1): 2u - 1 (exact in binary64)."""
    return 2.0 * uniform01(seed, stream, count, offset) - 1.0


def normal(seed: int, stream: int, count: int, offset: int = 0) -> np.ndarray:
    """Standard normal deviates, Box-Muller on consecutive uniform pairs."""
    u = uniform01(seed, stream, 2 * count, 2 * offset)
    u1 = 1.0 - u[0::2]          # (0, 1]
    u2 = u[1::2]
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def start_vector(n: int, seed: int = 0) -> np.ndarray:
    """The start vector dgetv0 draws (uniform[-1,1) from the given seed)."""
    return uniform_pm1(seed, STREAM_START, n)


def _coo_to_csr(n: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray,
                sum_duplicates: bool = True) -> CSR:
    """COO -> CSR with columns ascending in each row (duplicates summed when
    asked).  Uses scipy's compiled conversion."""
    from scipy.sparse import coo_matrix
    a = coo_matrix((np.asarray(vals, dtype=np.float64), (np.asarray(rows), np.asarray(cols))), shape=(n, n))
    a = a.tocsr()
    if sum_duplicates:
        a.sum_duplicates()
    a.sort_indices()
    return CSR(n, n, a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data.astype(np.float64))


def laplacian_2d(nx: int, ny: int | None = None) -> CSR:
    """5-point Dirichlet Laplacian on an nx x ny grid (diag 4, off-diagonals -1).

    Row of grid point (i, j) is i + nx*j.  Eigenvalues are
    4 - 2cos(a*pi/(nx+1)) - 2cos(b*pi/(ny+1)), a = 1..nx, b = 1..ny.
    """
    ny = nx if ny is None else ny
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    i, j = idx % nx, idx // nx
    rows, cols, vals = [idx], [idx], [np.full(n, 4.0)]
    for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (i + di >= 0) & (i + di < nx) & (j + dj >= 0) & (j + dj < ny)
        rows.append(idx[ok])
        cols.append(idx[ok] + di + nx * dj)
        vals.append(np.full(int(ok.sum()), -1.0))
    return _coo_to_csr(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals),
                       sum_duplicates=False)


def laplacian_2d_eigenvalues(nx: int, ny: int | None = None) -> np.ndarray:
    ny = nx if ny is None else ny
    a = np.arange(1, nx + 1)
    b = np.arange(1, ny + 1)
    ev = (4.0 - 2.0 * np.cos(a[:, None] * np.pi / (nx + 1))
          - 2.0 * np.cos(b[None, :] * np.pi / (ny + 1)))
    return np.sort(ev.ravel())


def laplacian_3d(N: int, shift_seed: int | None = 1, shift_max: float = 0.1) -> CSR:
    """7-point Dirichlet Laplacian on an N^3 grid (diag 6, off-diagonals -1),
    plus a per-row diagonal shift uniform[0, shift_max) from shift_seed
    (None: no shift).  Row of (i, j, k) is i + N*j + N*N*k."""
    n = N * N * N
    idx = np.arange(n, dtype=np.int64)
    i, j, k = idx % N, (idx // N) % N, idx // (N * N)
    diag = np.full(n, 6.0)
    if shift_seed is not None:
        diag = diag + shift_max * uniform01(shift_seed, STREAM_SHIFT, n)
    rows, cols, vals = [idx], [idx], [diag]
    for off, coord, step in ((-1, i, 1), (1, i, 1), (-1, j, N), (1, j, N), (-1, k, N * N), (1, k, N * N)):
        ok = (coord + off >= 0) & (coord + off < N)
        rows.append(idx[ok])
        cols.append(idx[ok] + off * step)
        vals.append(np.full(int(ok.sum()), -1.0))
    return _coo_to_csr(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals),
                       sum_duplicates=False)


def laplacian_3d_eigenvalues(N: int) -> np.ndarray:
    a = np.arange(1, N + 1)
    c = 2.0 - 2.0 * np.cos(a * np.pi / (N + 1))
    ev = c[:, None, None] + c[None, :, None] + c[None, None, :]
    return np.sort(ev.ravel())


def simple_dense(n: int = 16) -> np.ndarray:
    """K[i, j] = min(i, j) + 1, the matrix of the reference's data/simple.pp."""
    i = np.arange(n)
    return (np.minimum(i[:, None], i[None, :]) + 1).astype(np.float64)


def dense_to_csr(a: np.ndarray) -> CSR:
    n = a.shape[0]
    r, c = np.nonzero(a)
    return _coo_to_csr(n, r.astype(np.int64), c.astype(np.int64), a[r, c].astype(np.float64),
                       sum_duplicates=False)


def banded_random(n: int, half_bw: int, seed: int, problem: int = 0,
                  extra_frac: float = 0.10, extra_max: int = 8, diag_sigma: float = 2.0) -> CSR:
    """Symmetric banded random matrix (the batched workload's generator).

    Lower band entries (i, i-d), d = 1..half_bw, are N(0,1) and mirrored to
    the upper triangle; the diagonal is N(0, diag_sigma^2) (sigma 2, i.e.
    variance 4); a fraction extra_frac of rows carry 1..extra_max extra
    off-band entries (i, j), j uniform among columns outside the band, N(0,1),
    mirrored.  Entries landing on the same position are summed.  Draws use
    seed and the sub-stream 16*problem + k of STREAM_BAND.
    """
    s = lambda k: STREAM_BAND + 16 * (problem + 1) + k  # noqa: E731
    idx = np.arange(n, dtype=np.int64)
    rows, cols, vals = [idx], [idx], [diag_sigma * normal(seed, s(0), n)]
    band = normal(seed, s(1), n * half_bw).reshape(n, half_bw)
    for d in range(1, half_bw + 1):
        ok = idx >= d
        r = idx[ok]
        v = band[ok, d - 1]
        rows += [r, r - d]
        cols += [r - d, r]
        vals += [v, v]
    pick = uniform01(seed, s(2), n) < extra_frac
    er = idx[pick]
    cnt = 1 + (u64(seed, s(3), er.size) % np.uint64(extra_max)).astype(np.int64)
    total = int(cnt.sum())
    rr = np.repeat(er, cnt)
    # column outside [r - half_bw, r + half_bw]: draw among n - width candidates
    lo = np.maximum(rr - half_bw, 0)
    hi = np.minimum(rr + half_bw, n - 1)
    width = hi - lo + 1
    span = n - width
    ok = span > 0
    rr, lo, width, span = rr[ok], lo[ok], width[ok], span[ok]
    draw = (u64(seed, s(4), total)[ok] % span.astype(np.uint64)).astype(np.int64)
    cc = np.where(draw < lo, draw, draw + width)
    ev = normal(seed, s(5), total)[ok]
    rows += [rr, cc]
    cols += [cc, rr]
    vals += [ev, ev]
    return _coo_to_csr(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def batched_problem_sizes(count: int = 512, n_lo: int = 2000, n_hi: int = 200000,
                          bw_lo: int = 2, bw_hi: int = 16, seed: int = 3):
    """Sizes and half-bandwidths of the batched workload: n log-uniform in
    [n_lo, n_hi], half-bandwidth uniform in {bw_lo..bw_hi}."""
    u = uniform01(seed, STREAM_BAND, count)
    n = np.floor(np.exp(np.log(n_lo) + u * (np.log(n_hi) - np.log(n_lo)))).astype(np.int64)
    bw = bw_lo + (u64(seed, STREAM_BAND + 1, count) % np.uint64(bw_hi - bw_lo + 1)).astype(np.int64)
    return n, bw


def _count_le(cdf: np.ndarray, x: np.ndarray) -> np.ndarray:
    """searchsorted(cdf, uniform01 of the raw draws x, side="right") for a
    sorted cdf in [0, 1], through a bucket index: bucket b = x >> (64 - k)
    holds the draws in [b 2^-k, (b+1) 2^-k), lo[b] counts the cdf entries
    below the bucket, and the few entries inside it are compared directly.
    Exactly the same counts as the binary search, several times fewer
    random memory accesses."""
    k = max(10, min(26, int(np.ceil(np.log2(max(cdf.size, 2)))) + 2))
    edges = np.arange((1 << k) + 1, dtype=np.float64) * (2.0 ** -k)
    lo = np.searchsorted(cdf, edges, side="right")
    span = int(np.diff(lo).max()) if lo.size > 1 else 0
    u = (x >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    base = lo[(x >> np.uint64(64 - k)).astype(np.int64)]
    padded = np.concatenate([cdf, np.full(span + 1, np.inf)])
    out = base.copy()
    for t in range(span):
        out += padded[base + t] <= u
    return out


def chung_lu_normalized(n: int, gamma: float = 2.5, mean_degree: float = 32.0, seed: int = 2) -> CSR:
    """Symmetric normalised adjacency D^-1/2 A D^-1/2 of a Chung-Lu graph.

    Expected degrees w_i = C (i + i0)^(-1/(gamma-1)); C fixes the mean degree
    and i0 caps the largest weight at sqrt(n * mean_degree) (the structural
    cutoff that keeps w_i w_j / sum(w) <= 1).  round(n * mean_degree / 2)
    edges are drawn with both endpoints i.i.d. proportional to w; self-loops
    are dropped and multi-edges merged (unweighted adjacency).  Every
    connected component other than the largest is then joined to the largest
    by one edge (between draws from each), and isolated vertices likewise, so
    the graph is connected and eigenvalue 1 is simple.
    """
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    expo = 1.0 / (gamma - 1.0)
    target = np.sqrt(n * mean_degree)
    i = np.arange(n, dtype=np.float64)

    def weights(i0):
        w = (i + i0) ** (-expo)
        return w * (mean_degree * n / w.sum())

    def first_weight(i0):            # weights(i0)[0] without scaling the whole array
        w = (i + i0) ** (-expo)
        return w[0] * (mean_degree * n / w.sum())

    lo, hi = 1e-3, float(n)
    for _ in range(100):     # bisection on i0 so that w_0 = target
        mid = np.sqrt(lo * hi)
        nlo, nhi = (mid, hi) if first_weight(mid) > target else (lo, mid)
        if nlo == lo and nhi == hi:  # fixed point: the remaining steps change nothing
            break
        lo, hi = nlo, nhi
    w = weights(hi)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    m = int(round(n * mean_degree / 2))
    ua = u64(seed, STREAM_GRAPH, m)
    ub = u64(seed, STREAM_GRAPH, m, offset=m)
    a = np.minimum(_count_le(cdf, ua), n - 1)
    b = np.minimum(_count_le(cdf, ub), n - 1)
    keep = a != b
    a, b = a[keep], b[keep]
    # both orientations in one conversion (duplicates summed, then unit weights)
    adj = coo_matrix((np.ones(2 * a.size), (np.concatenate([a, b]), np.concatenate([b, a]))),
                     shape=(n, n)).tocsr()
    adj.data[:] = 1.0
    ncomp, labels = connected_components(adj, directed=False)
    if ncomp > 1:
        sizes = np.bincount(labels)
        giant = int(np.argmax(sizes))
        giant_nodes = np.nonzero(labels == giant)[0]
        order = np.argsort(labels, kind="stable")
        starts = np.searchsorted(labels[order], np.arange(ncomp))
        others = np.array([c for c in range(ncomp) if c != giant], dtype=np.int64)
        rep = order[starts[others]]                       # first vertex of each component
        pick = (u64(seed, STREAM_GRAPH + 1, others.size) % np.uint64(giant_nodes.size)).astype(np.int64)
        tgt = giant_nodes[pick]
        extra = coo_matrix((np.ones(2 * rep.size), (np.concatenate([rep, tgt]), np.concatenate([tgt, rep]))),
                           shape=(n, n)).tocsr()
        adj = adj + extra
        adj.data[:] = 1.0
    adj.sort_indices()
    deg = np.diff(adj.indptr).astype(np.float64)
    dinv = 1.0 / np.sqrt(deg)
    rows = np.repeat(np.arange(n), np.diff(adj.indptr))
    vals = dinv[rows] * dinv[adj.indices]
    return CSR(n, n, adj.indptr.astype(np.int32), adj.indices.astype(np.int32), vals.astype(np.float64))


def lower_triangle(m: CSR) -> CSR:
    """The symmetric-lower storage of a general symmetric CSR (col <= row),
    the form the reference's readers produce for symmetric files."""
    rows = np.repeat(np.arange(m.n, dtype=np.int64), np.diff(m.row_ptr))
    keep = m.col <= rows
    r, c, v = rows[keep], m.col[keep].astype(np.int64), m.val[keep]
    return _coo_to_csr(m.n, r, c, v, sum_duplicates=False)


def to_scipy(m: CSR):
    from scipy.sparse import csr_matrix
    return csr_matrix((m.val, m.col, m.row_ptr), shape=(m.n, m.ncols))
