"""Seeded synthetic SPD matrices for the supernodal Cholesky workloads.

Every generator is deterministic across machines (x86_64 and aarch64): values
are built only from IEEE-754 +, -, *, / and sqrt (each correctly rounded in
numpy's elementwise ufuncs) and a counter-based splitmix64 stream, never from
libm transcendental functions whose last bit can differ between platforms.
Log-uniform samples use :func:`det_exp`, an exp written here from its
definition (Cody-Waite range reduction + Taylor polynomial).

Matrices are returned as the lower triangle in compressed-column form with
sorted row indices (CHOLMOD's ``stype = -1`` symmetric-lower convention,
cholmod.h:1168-1206): ``(n, Ap int64[n+1], Ai int64[nnz], Ax float64[nnz])``.

Workloads (each a stand-in with the reference benchmark's shapes, sizes and
value distributions; no public matrix collection is read):
  * ``laplace2d(nx, ny, ...)`` 5-point Dirichlet Laplacian, constant or
    log-uniform edge coefficients, optional diagonal shift.
  * ``laplace3d(nx, ny, nz, ...)`` 7-point Dirichlet Laplacian.
  * ``elastic27(m, seed)`` 27-point stencil with 3 unknowns per grid node.
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, count, offset=0):
    """``count`` outputs of the splitmix64 stream of ``seed`` (uint64)."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, count, offset=0):
    """Uniform doubles in [0, 1) with 53 random bits."""
    z = splitmix64(seed, count, offset) >> np.uint64(11)
    return z.astype(np.float64) * (1.0 / 9007199254740992.0)


_LN2_HI = 6.93147180369123816490e-01   # ln 2 split so that k*_LN2_HI is exact
_LN2_LO = 1.90821492927058770002e-10


def det_exp(x):
    """exp(x) from +,-,* only: x = k ln2 + r, |r| <= ln2/2, Taylor to r^17."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * (1.0 / 0.6931471805599453))
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.ones_like(r)
    for j in range(17, 0, -1):          # Horner: 1 + r/1 (1 + r/2 (1 + ...))
        p = 1.0 + (r / float(j)) * p
    return np.ldexp(p, k.astype(np.int64))


def det_log(x):
    """ln(x) of a positive scalar from +,-,*,/ only: x = m 2^e with m in
    [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)) summed to convergence."""
    m, e = np.frexp(np.float64(x))
    if m < 0.7071067811865476:
        m, e = m * 2.0, e - 1
    t = (m - 1.0) / (m + 1.0)
    t2, term, acc = t * t, t, 0.0
    for j in range(1, 80, 2):
        acc = acc + term / j
        term = term * t2
    return float(2.0 * acc + e * _LN2_HI + e * _LN2_LO)


def log_uniform(lo, hi, u):
    """Map uniform u in [0,1) to log-uniform values in [lo, hi]."""
    a = det_log(lo)
    b = det_log(hi)
    return det_exp(a + u * (b - a))


def _csc_lower(n, rows, cols, vals):
    """Sum duplicates of (rows >= cols) triplets into sorted lower CSC."""
    keep = rows >= cols
    rows, cols, vals = rows[keep], cols[keep], vals[keep]
    order = np.lexsort((rows, cols))
    rows, cols, vals = rows[order], cols[order], vals[order]
    key = cols * np.int64(n) + rows
    uniq, start = np.unique(key, return_index=True)
    sums = np.add.reduceat(vals, start) if len(vals) else vals
    Ai = (uniq % n).astype(np.int64)
    Aj = (uniq // n).astype(np.int64)
    Ap = np.zeros(n + 1, dtype=np.int64)
    np.add.at(Ap, Aj + 1, 1)
    Ap = np.cumsum(Ap).astype(np.int64)
    return n, Ap, Ai, np.ascontiguousarray(sums, dtype=np.float64)


def _grid_laplacian(dims, coef, shift):
    """Dirichlet graph Laplacian on a box grid; ``coef[d]`` are the edge
    conductivities of direction d, shape dims with dims[d] + 1 along axis d
    (edges to the ghost layer on both faces included)."""
    dims = tuple(int(v) for v in dims)
    n = int(np.prod(dims))
    idx = np.arange(n, dtype=np.int64).reshape(dims[::-1]).transpose()  # x fastest
    diag = np.full(dims, float(shift))
    rows, cols, vals = [], [], []
    for d, c in enumerate(coef):
        lo = [slice(None)] * len(dims)
        hi = [slice(None)] * len(dims)
        lo[d] = slice(0, dims[d])       # edge before node
        hi[d] = slice(1, dims[d] + 1)   # edge after node
        diag = diag + c[tuple(lo)] + c[tuple(hi)]
        a = [slice(None)] * len(dims)
        b = [slice(None)] * len(dims)
        a[d] = slice(0, dims[d] - 1)
        b[d] = slice(1, dims[d])
        inner = [slice(None)] * len(dims)
        inner[d] = slice(1, dims[d])
        i = idx[tuple(b)].ravel(order="F")
        j = idx[tuple(a)].ravel(order="F")
        v = -c[tuple(inner)].ravel(order="F")
        rows.append(i)
        cols.append(j)
        vals.append(v)
    rows.append(idx.ravel(order="F"))
    cols.append(idx.ravel(order="F"))
    vals.append(diag.ravel(order="F"))
    return _csc_lower(n, np.concatenate(rows), np.concatenate(cols),
                      np.concatenate(vals))


def _edge_coefs(dims, seed, lo, hi):
    coef = []
    offset = 0
    for d in range(len(dims)):
        shp = list(dims)
        shp[d] += 1
        cnt = int(np.prod(shp))
        u = uniform01(seed, cnt, offset)
        offset += cnt
        coef.append(log_uniform(lo, hi, u).reshape(shp[::-1]).transpose())
    return coef


def laplace2d(nx, ny=None, seed=None, lo=1e-2, hi=1e2, shift=0.0):
    """2D 5-point Laplacian; constant unit coefficients when seed is None."""
    ny = nx if ny is None else ny
    dims = (nx, ny)
    if seed is None:
        coef = [np.ones((nx + 1, ny)), np.ones((nx, ny + 1))]
    else:
        coef = _edge_coefs(dims, seed, lo, hi)
    return _grid_laplacian(dims, coef, shift)


def laplace3d(nx, ny=None, nz=None, seed=None, lo=1e-2, hi=1e2, shift=0.0):
    """3D 7-point Laplacian; constant unit coefficients when seed is None."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    dims = (nx, ny, nz)
    if seed is None:
        coef = [np.ones((nx + 1, ny, nz)), np.ones((nx, ny + 1, nz)),
                np.ones((nx, ny, nz + 1))]
    else:
        coef = _edge_coefs(dims, seed, lo, hi)
    return _grid_laplacian(dims, coef, shift)


def magnetic_laplacian(dims, seed=11, lo=1e-1, hi=1e1, shift=1e-2, diag_imag=0.0):
    """Hermitian positive definite test matrix: the graph Laplacian of a box
    grid (5- or 7-point, Dirichlet, log-uniform conductivities) whose
    off-diagonal entries carry unit phases -- the discrete magnetic
    Laplacian -- plus shift on the diagonal.  A phase is the unit complex
    number ((1 - t^2) + 2 t i) / (1 + t^2), t uniform in [-1, 1), so that
    only correctly rounded arithmetic is used and the values are the same on
    every platform.  diag_imag puts that imaginary part on every diagonal
    entry (the factorization ignores it).  Returns (n, Ap, Ai, Ax) of the
    lower triangle with complex Ax."""
    dims = tuple(int(v) for v in dims)
    n, Ap, Ai, Ax = _grid_laplacian(dims, _edge_coefs(dims, seed, lo, hi), shift)
    col = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    off = Ai != col
    t = 2.0 * uniform01(seed + 101, int(off.sum())) - 1.0
    den = 1.0 + t * t
    z = np.ones(len(Ax), dtype=np.complex128)
    z[off] = (1.0 - t * t) / den + 1j * (2.0 * t / den)
    Axc = Ax * z
    Axc[~off] += 1j * diag_imag
    return n, Ap, Ai, Axc


def _rotations(u):
    """Rotation matrices from unit quaternions built from 4 uniforms each."""
    q = 2.0 * u.reshape(-1, 4) - 1.0
    nrm = np.sqrt(((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2])
                  + q[:, 3] * q[:, 3])
    nrm[nrm == 0] = 1.0
    w, x, y, z = (q / nrm[:, None]).T
    R = np.empty((len(w), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _spd_blocks(seed, count, offset, lo=0.1, hi=10.0):
    """``count`` random 3x3 SPD blocks Q diag(lam) Q', lam log-uniform."""
    u = uniform01(seed, 7 * count, offset)
    lam = log_uniform(lo, hi, u[:3 * count]).reshape(count, 3)
    Q = _rotations(u[3 * count:])
    B = np.zeros((count, 3, 3))
    for i in range(3):              # explicit sums: fixed order on any platform
        for l in range(3):
            acc = Q[:, i, 0] * lam[:, 0] * Q[:, l, 0]
            acc = acc + Q[:, i, 1] * lam[:, 1] * Q[:, l, 1]
            acc = acc + Q[:, i, 2] * lam[:, 2] * Q[:, l, 2]
            B[:, i, l] = acc
    return 0.5 * (B + B.transpose(0, 2, 1))


def elastic27(m, seed=2, dof=3, margin=1e-6):
    """27-point stencil on an m^3 grid with 3 unknowns per node.

    Each coupling between two neighbouring nodes is minus a random 3x3 SPD
    block (eigenvalues log-uniform in [0.1, 10]); each node's own block is a
    random SPD block whose diagonal is then raised, where needed, so that
    every row is strictly diagonally dominant by ``margin``.
    """
    assert dof == 3
    nn = m ** 3
    n = nn * 3
    node = np.arange(nn, dtype=np.int64).reshape(m, m, m).transpose()  # x fastest
    offs = [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1)
            for dx in (-1, 0, 1) if (dx, dy, dz) > (0, 0, 0)]
    # forward neighbour pairs (13 directions), lexicographically positive
    pi, pj = [], []
    for (dx, dy, dz) in offs:
        xs = slice(max(0, -dx), m - max(0, dx))
        ys = slice(max(0, -dy), m - max(0, dy))
        zs = slice(max(0, -dz), m - max(0, dz))
        a = node[xs, ys, zs]
        b = node[slice(xs.start + dx, xs.stop + dx), slice(ys.start + dy, ys.stop + dy),
                 slice(zs.start + dz, zs.stop + dz)]
        pi.append(a.ravel(order="F"))
        pj.append(b.ravel(order="F"))
    pi = np.concatenate(pi)
    pj = np.concatenate(pj)
    npair = len(pi)
    Boff = -_spd_blocks(seed, npair, 0)
    Bdiag = _spd_blocks(seed, nn, 7 * npair)
    # row sums of |off-diagonal| for diagonal dominance
    aB = np.abs(Boff)
    rows_abs = (aB[:, :, 0] + aB[:, :, 1]) + aB[:, :, 2]     # row sums of |B|
    cols_abs = (aB[:, 0, :] + aB[:, 1, :]) + aB[:, 2, :]     # row sums of |B'|
    absoff = np.zeros((nn, 3))
    np.add.at(absoff, pi, rows_abs)
    np.add.at(absoff, pj, cols_abs)
    aD = np.abs(Bdiag)
    own = np.stack([aD[:, 0, 1] + aD[:, 0, 2], aD[:, 1, 0] + aD[:, 1, 2],
                    aD[:, 2, 0] + aD[:, 2, 1]], axis=1)
    need = absoff + own + margin
    d = np.stack([Bdiag[:, 0, 0], Bdiag[:, 1, 1], Bdiag[:, 2, 2]], axis=1)
    newd = np.where(d >= need, d, need)
    Bdiag = Bdiag.copy()
    for r in range(3):
        Bdiag[:, r, r] = newd[:, r]
    # assemble triplets: node block (I,J) -> rows 3I+r, cols 3J+c
    r3 = np.arange(3)
    rows, cols, vals = [], [], []
    # off-diagonal blocks, both (i,j) and (j,i) = block^T (symmetric blocks)
    for (I, J, B) in ((pi, pj, Boff), (pj, pi, Boff.transpose(0, 2, 1))):
        rows.append((3 * I[:, None, None] + r3[None, :, None]).repeat(3, axis=2).ravel())
        cols.append((3 * J[:, None, None] + r3[None, None, :]).repeat(3, axis=1).ravel())
        vals.append(B.ravel())
    I = np.arange(nn, dtype=np.int64)
    rows.append((3 * I[:, None, None] + r3[None, :, None]).repeat(3, axis=2).ravel())
    cols.append((3 * I[:, None, None] + r3[None, None, :]).repeat(3, axis=1).ravel())
    vals.append(Bdiag.ravel())
    return _csc_lower(n, np.concatenate(rows).astype(np.int64),
                      np.concatenate(cols).astype(np.int64), np.concatenate(vals))


def rhs(n, nrhs, seed):
    """Right-hand sides with entries i.i.d. uniform in [-1, 1], column-major."""
    return (2.0 * uniform01(seed, n * nrhs) - 1.0).reshape(nrhs, n).T.copy(order="F")


def full_from_lower(n, Ap, Ai, Ax):
    """Both triangles (CSC) of a symmetric matrix stored as its lower part."""
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    off = Ai != cols
    r = np.concatenate([Ai, cols[off]])
    c = np.concatenate([cols, Ai[off]])
    v = np.concatenate([Ax, Ax[off]])
    order = np.lexsort((r, c))
    r, c, v = r[order], c[order], v[order]
    Fp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(Fp, c + 1, 1)
    return np.cumsum(Fp).astype(np.int64), r.astype(np.int64), v


def digest(*arrays):
    """SHA-256 over the raw bytes of the given arrays (fixture fingerprints)."""
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def batch_sides(seed=3, count=8, lo=16, hi=96):
    """``count`` distinct grid sides drawn uniformly from [lo, hi] (splitmix64
    stream of ``seed``, first draws kept, repeats skipped)."""
    sides, off = [], 0
    while len(sides) < count:
        u = uniform01(seed, 64, off)
        off += 64
        for v in u:
            s = lo + int(v * (hi - lo + 1))
            if s not in sides:
                sides.append(s)
                if len(sides) == count:
                    break
    return sides


def batch_system(index, side, seed=3, lo=0.1, hi=10.0):
    """System ``index`` of the batched workload: 2D 5-point Laplacian on a
    side x side grid with log-uniform edge coefficients in [lo, hi]."""
    return laplace2d(side, side, seed=(seed << 32) + index + 1, lo=lo, hi=hi)


def grid_nd_perm(dims, leaf=16):
    """Geometric nested-dissection ordering of a box grid (x fastest, as the
    grid generators number nodes): recursive bisection across the longest
    side, each separator plane ordered after both halves.  Returns Perm with
    Perm[k] = original index of the k-th pivot."""
    dims = tuple(int(v) for v in dims)
    strides = np.cumprod((1,) + dims[:-1]).astype(np.int64)
    out = []
    stack = [(tuple(0 for _ in dims), dims)]
    # explicit post-order: (box, state) with state 0 = expand, 1 = emit separator
    work = [("box", (0,) * len(dims), dims)]
    while work:
        kind, lo, sz = work.pop()
        if kind == "sep" or int(np.prod(sz)) <= leaf or max(sz) <= 2:
            grids = np.meshgrid(*[np.arange(l, l + s) for l, s in zip(lo, sz)], indexing="ij")
            ids = sum(g.astype(np.int64) * st for g, st in zip(grids, strides))
            out.append(ids.ravel(order="F"))
            continue
        d = int(np.argmax(sz))
        m = sz[d] // 2
        left_sz = list(sz); left_sz[d] = m
        right_lo = list(lo); right_lo[d] = lo[d] + m + 1
        right_sz = list(sz); right_sz[d] = sz[d] - m - 1
        sep_lo = list(lo); sep_lo[d] = lo[d] + m
        sep_sz = list(sz); sep_sz[d] = 1
        # pushed in reverse: left, right, then the separator last
        work.append(("sep", tuple(sep_lo), tuple(sep_sz)))
        if right_sz[d] > 0:
            work.append(("box", tuple(right_lo), tuple(right_sz)))
        if m > 0:
            work.append(("box", lo, tuple(left_sz)))
    del stack
    return np.concatenate(out).astype(np.int64)


def batch_layout(nsys=4096, seed=3, npat=8, lo=16, hi=96):
    """The batched workload's systems: ``npat`` distinct grid sides
    (batch_sides) and, for each of ``nsys`` systems, the index of its side
    (uniform over the sides, splitmix64 stream of ``seed`` + 1)."""
    sides = batch_sides(seed, npat, lo, hi)
    u = uniform01(seed + 1, nsys, 0)
    pat = np.minimum((u * npat).astype(np.int32), npat - 1)
    return sides, pat


def block_diag_lower(mats):
    """Lower-triangular CSC of diag(A_0, A_1, ...) from (n, Ap, Ai, Ax) tuples."""
    n = sum(m[0] for m in mats)
    nnz = sum(int(m[1][-1]) for m in mats)
    Ap = np.zeros(n + 1, dtype=np.int64)
    Ai = np.empty(nnz, dtype=np.int64)
    Ax = np.empty(nnz, dtype=np.float64)
    c0 = p0 = 0
    for (ni, p, i, x) in mats:
        k = int(p[-1])
        Ap[c0 + 1:c0 + ni + 1] = p0 + p[1:]
        Ai[p0:p0 + k] = c0 + i
        Ax[p0:p0 + k] = x
        c0 += ni
        p0 += k
    return n, Ap, Ai, Ax


# Named workloads (the benchmark configurations; parity-test cases)
CONFIGS = {
    "c1": dict(kind="laplace2d", args=dict(nx=100, shift=1e-3), ordering="amd",
               rhs_seed=0, nrhs=1),
    "c2": dict(kind="laplace3d", args=dict(nx=64, seed=1, lo=1e-2, hi=1e2),
               ordering="metis", rhs_seed=1, nrhs=1),
    "c3": dict(kind="elastic27", args=dict(m=40, seed=2), ordering="metis",
               rhs_seed=2, nrhs=1),
}


def config_matrix(name):
    c = CONFIGS[name]
    gen = {"laplace2d": laplace2d, "laplace3d": laplace3d, "elastic27": elastic27}[c["kind"]]
    return gen(**c["args"])
