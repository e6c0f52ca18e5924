"""Seeded synthetic sparse matrices for the benchmark workloads and tests.

The reference evaluates on SuiteSparse / PyG graphs that are not available
offline; these generators stand in for them with the shapes, sizes and value
distributions of the five workloads:

  uniform_c1     512 x 512, ~2 % uniform positions, U[-1, 1] values
  rmat_c2        R-MAT 16384 (a, b, c, d = .57, .19, .19, .05), 131072 edges
                 drawn, symmetrised, duplicates merged, N(0, 1) values
  rmat_batch     256 R-MAT matrices, rows log-uniform in [256, 8192],
                 average degree U[4, 32], U[-1, 1] values
  rmat_c4        R-MAT 65536, average degree 32
  chung_lu_c5    Chung-Lu power law (exponent 2.1, mean degree 20), 262144
                 nodes, symmetric-normalised weights D^-1/2 A D^-1/2
  vnm_structured a matrix already in full V:2:M form (every V x M block
                 keeps 4 columns, 2 nonzeros a row among them)

All return (nrows, row, col, val) with (row, col) unique and sorted, which is
the order the Matrix Market reader leaves a matrix in.
"""
import numpy as np


def _nonzero_values(rng, n, kind):
    if kind == "uniform":
        v = rng.uniform(-1.0, 1.0, n).astype(np.float32)
        # a value that "%.2f" prints as 0.00 would turn into an explicit zero
        # after the reference's text round trip; redraw those
        bad = np.abs(v) < 0.005
        while bad.any():
            v[bad] = rng.uniform(-1.0, 1.0, int(bad.sum())).astype(np.float32)
            bad = np.abs(v) < 0.005
        return v
    if kind == "normal":
        return rng.standard_normal(n).astype(np.float32)
    raise ValueError(kind)


def uniform(R, density, seed, values="uniform"):
    """Distinct uniformly random (row, col) positions."""
    rng = np.random.default_rng(seed)
    nnz = int(round(R * R * density))
    idx = np.sort(rng.choice(R * R, nnz, replace=False))
    row = (idx // R).astype(np.int32)
    col = (idx % R).astype(np.int32)
    return R, row, col, _nonzero_values(rng, nnz, values)


def uniform_c1(seed=0):
    return uniform(512, 0.02, seed)


def rmat_edges(scale, nedges, rng, a=0.57, b=0.19, c=0.19):
    r = np.zeros(nedges, np.int64)
    q = np.zeros(nedges, np.int64)
    for _ in range(scale):
        u = rng.random(nedges)
        rbit = u >= a + b
        cbit = ((u >= a) & (u < a + b)) | (u >= a + b + c)
        r = 2 * r + rbit
        q = 2 * q + cbit
    return r, q


def rmat(scale, nedges, seed, values="normal", R=None):
    """Symmetrised R-MAT graph, self-loops kept, duplicates merged."""
    rng = np.random.default_rng(seed)
    r, q = rmat_edges(scale, nedges, rng)
    n = 1 << scale
    if R is not None and R < n:  # fold ids into [0, R) for non power-of-two sizes
        r %= R
        q %= R
        n = R
    key = np.unique(np.concatenate([r * n + q, q * n + r]))
    row = (key // n).astype(np.int32)
    col = (key % n).astype(np.int32)
    return n, row, col, _nonzero_values(rng, len(key), values)


def rmat_c2(seed=0):
    return rmat(14, 131072, seed, "normal")


def rmat_batch(count=256, seed=1000, lo=256, hi=8192):
    """The batched workload: row counts log-uniform in [lo, hi], degree U[4, 32]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        R = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        deg = rng.uniform(4.0, 32.0)
        scale = int(np.ceil(np.log2(R)))
        nedges = max(1, int(R * deg / 2))
        out.append(rmat(scale, nedges, seed + 1 + i, "uniform", R=R))
    return out


def rmat_c4(seed=0):
    return rmat(16, 65536 * 16, seed, "normal")


def chung_lu(n, exponent, mean_degree, seed):
    """Chung-Lu graph with power-law expected degrees, symmetric-normalised."""
    rng = np.random.default_rng(seed)
    i = np.arange(1, n + 1, dtype=np.float64)
    w = i ** (-1.0 / (exponent - 1.0))
    w *= mean_degree * n / w.sum()
    m = int(mean_degree * n / 2)
    p = w / w.sum()
    u = rng.choice(n, m, p=p)
    v = rng.choice(n, m, p=p)
    key = np.unique(np.concatenate([u * n + v, v * n + u]))
    row = (key // n).astype(np.int64)
    col = (key % n).astype(np.int64)
    deg = np.bincount(row, minlength=n).astype(np.float64)
    dinv = np.where(deg > 0, 1.0 / np.sqrt(np.maximum(deg, 1.0)), 0.0)
    val = (dinv[row] * dinv[col]).astype(np.float32)
    return n, row.astype(np.int32), col.astype(np.int32), val


def chung_lu_c5(seed=0):
    return chung_lu(262144, 2.1, 20.0, seed)


# the six ways to keep 2 of 4 columns
_PAIRS_OF_4 = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], np.int64)


def vnm_structured(R, M=8, V=128, seed=0):
    """A matrix already in full V:2:M form, the operand V:N:M sparsity is
    made for (a pruned weight matrix): in every block of V rows x M columns
    4 columns are kept and every row holds 2 nonzeros among them, so each
    block has 2V nonzeros and the density is 2/M.  N(0, 1) values; (row,
    col) sorted.  R must be a multiple of V and of M."""
    assert R % V == 0 and R % M == 0 and M >= 4
    rng = np.random.default_rng(seed)
    nbr, nseg = R // V, R // M
    keep = np.sort(np.argsort(rng.random((nbr, nseg, M)), axis=-1)[..., :4], axis=-1)  # [nbr][nseg][4]
    combo = rng.integers(0, 6, (R, nseg), dtype=np.int8)
    pick = _PAIRS_OF_4[combo]                                                            # [R][nseg][2]
    k = keep[np.arange(R)[:, None] // V, np.arange(nseg)[None, :]]                       # [R][nseg][4]
    sel = np.take_along_axis(k, pick, axis=-1)                                          # [R][nseg][2], ascending
    col = (np.arange(nseg, dtype=np.int64)[None, :, None] * M + sel).reshape(-1).astype(np.int32)
    row = np.repeat(np.arange(R, dtype=np.int32), nseg * 2)
    return R, row, col, rng.standard_normal(len(row), dtype=np.float32)


def write_mtx(path, nrows, row, col, val, field="real"):
    """Matrix Market writer for test inputs ("%.6g" values, 1-based)."""
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate %s general\n" % field)
        f.write("%d %d %d\n" % (nrows, nrows, len(row)))
        if field == "pattern":
            for r, c in zip(row.tolist(), col.tolist()):
                f.write("%d %d\n" % (r + 1, c + 1))
        else:
            for r, c, v in zip(row.tolist(), col.tolist(), val.tolist()):
                f.write("%d %d %.6g\n" % (r + 1, c + 1, v))
