"""
CPU oracle for the single-site TDVP / DMRG path.

TEST INFRASTRUCTURE ONLY. This module is the checker against which the GPU
engine in ``pytenet_gb300`` is compared. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and its
``--impl reference`` arm) may import it. The product path never calls it.

It restates, in NumPy, the algorithm of PyTeNet (cmendl/pytenet) for the
single-site path. Every function names the reference file and lines it
follows (paths relative to the reference project root). The restatement
keeps the reference's order of NumPy operations so that, on the same BLAS,
results agree bit for bit; the golden fixtures under ``tests/golden/`` pin it
against outputs of the reference itself.

Objects passed in are duck-typed: anything with ``.a`` (list of ndarrays),
``.qsite`` and ``.qbonds`` works as an MPS, anything with ``.a``, ``.qsite``,
``.qbonds`` works as an MPO (both the reference's classes and
``pytenet_gb300``'s).
"""

import warnings
import numpy as np

__all__ = [
    "crandn", "qnumber_outer_sum", "qnumber_flatten", "is_qsparse",
    "enforce_qsparsity", "common_qnumbers", "sort_by_qnumbers", "block_sparse_qr",
    "OMPS", "random_mps", "local_orthonormalize_left_qr", "local_orthonormalize_right_qr",
    "orthonormalize", "mps_to_vector", "mpo_to_matrix", "mps_vdot", "mps_norm",
    "env_step_right", "env_step_left", "compute_right_operator_blocks",
    "apply_local_hamiltonian", "apply_local_bond_contraction",
    "mpo_inner_product", "mpo_average",
    "lanczos_iteration", "eigh_tridiag", "expm_krylov", "eigh_krylov",
    "tdvp_singlesite", "dmrg_singlesite", "compress_svd", "compress_density",
    "block_sparse_eigh",
]


# ---------------------------------------------------------------------------
# random numbers -- pytenet/util.py:10-17
# ---------------------------------------------------------------------------

def crandn(size, rng):
    """Standard complex normal samples: all real parts are drawn first, then all
    imaginary parts, scaled by 1/sqrt(2) (pytenet/util.py:10-17)."""
    re = rng.normal(size=size)
    im = rng.normal(size=size)
    return (re + 1j*im) / np.sqrt(2)


# ---------------------------------------------------------------------------
# quantum-number bookkeeping -- pytenet/block_sparse_util.py:13-103
# ---------------------------------------------------------------------------

def qnumber_outer_sum(qnums):
    """Outer sum of quantum-number lists (block_sparse_util.py:13-30)."""
    if len(qnums) == 0:
        return np.array(0)
    out = qnums[0]
    for q in qnums[1:]:
        out = np.add.outer(out, q)
    return out


def qnumber_flatten(qnums):
    """Flattened outer sum (block_sparse_util.py:40-44)."""
    return qnumber_outer_sum(qnums).reshape(-1)


def common_qnumbers(q0, q1):
    """Sorted common quantum numbers (block_sparse_util.py:33-37)."""
    return np.intersect1d(q0, q1)


def is_qsparse(a, qnums):
    """True if all entries whose quantum numbers do not sum to zero vanish
    (block_sparse_util.py:47-53)."""
    mask = qnumber_outer_sum(qnums)
    return not np.any(np.where(mask == 0, 0, a))


def enforce_qsparsity(a, qnums):
    """Zero all entries whose quantum numbers do not sum to zero, in place
    (block_sparse_util.py:56-64; vectorised, same result as the element loop)."""
    mask = qnumber_outer_sum(qnums)
    a[np.broadcast_to(mask != 0, a.shape)] = 0


def sort_by_qnumbers(a, q0, q1):
    """Stable sort of rows and columns by quantum number
    (block_sparse_util.py:67-92)."""
    q0 = np.asarray(q0)
    q1 = np.asarray(q1)
    idx0 = np.argsort(q0, kind="mergesort")
    idx1 = np.argsort(q1, kind="mergesort")
    if np.any(idx0 - np.arange(len(idx0))):
        q0 = q0[idx0]
        a = a[idx0, :]
    if np.any(idx1 - np.arange(len(idx1))):
        q1 = q1[idx1]
        a = a[:, idx1]
    return a, (idx0, q0), (idx1, q1)


def _qslice(qn, qnums):
    """First..last index of `qn` in sorted `qnums` (block_sparse_util.py:95-103)."""
    where = np.where(qnums == qn)[0]
    return slice(where[0], where[-1] + 1)


def block_sparse_qr(a, q0, q1):
    """Block-wise reduced QR respecting quantum numbers
    (block_sparse_util.py:106-180)."""
    a = np.asarray(a)
    assert a.ndim == 2
    assert len(q0) == a.shape[0] and len(q1) == a.shape[1]
    assert is_qsparse(a, [q0, -q1])
    qis = common_qnumbers(q0, q1)
    if len(qis) == 0:
        # no common quantum number: dummy bond of dimension 1 (lines 124-135)
        assert np.linalg.norm(a) == 0
        q = np.zeros((a.shape[0], 1), dtype=a.dtype)
        r = np.zeros((1, a.shape[1]), dtype=a.dtype)
        q[0, 0] = 1
        return q, r, q0[:1]
    a, (idx0, q0), (idx1, q1) = sort_by_qnumbers(a, q0, q1)
    kmax = min(a.shape)
    q = np.zeros((a.shape[0], kmax), dtype=a.dtype)
    r = np.zeros((kmax, a.shape[1]), dtype=a.dtype)
    qinterm = np.zeros(kmax, dtype=q0.dtype)
    k = 0
    for qn in qis:
        rs = _qslice(qn, q0)
        cs = _qslice(qn, q1)
        qb, rb = np.linalg.qr(a[rs, cs], mode="reduced")
        k0, k = k, k + qb.shape[1]
        q[rs, k0:k] = qb
        r[k0:k, cs] = rb
        qinterm[k0:k] = qn
    assert k <= kmax
    q = q[:, :k]
    r = r[:k, :]
    qinterm = qinterm[:k]
    if np.any(idx0 - np.arange(len(idx0))):
        q = q[np.argsort(idx0), :]
    if np.any(idx1 - np.arange(len(idx1))):
        r = r[:, np.argsort(idx1)]
    return q, r, qinterm


# ---------------------------------------------------------------------------
# MPS container and gauge operations -- pytenet/mps.py
# ---------------------------------------------------------------------------

class OMPS:
    """Minimal MPS container (pytenet/mps.py:14-71): list `a` of
    (b[i], d, b[i+1]) tensors plus integer `qsite` / `qbonds`."""

    def __init__(self, qsite, qbonds, a=None):
        self.qsite = np.asarray(qsite)
        self.qbonds = [np.asarray(q) for q in qbonds]
        self.a = a if a is not None else [None] * (len(qbonds) - 1)

    @property
    def nsites(self):
        return len(self.a)

    @property
    def bond_dims(self):
        return [x.shape[0] for x in self.a] + [self.a[-1].shape[2]]


def random_mps(qsite, qbonds, rng, real=False):
    """Random MPS with the same draw order as `MPS(..., fill="random")`
    (mps.py:49-71): site by site, crandn((b_i, d, b_{i+1})) / sqrt(b_i d b_{i+1}),
    then the quantum-number mask."""
    psi = OMPS(qsite, qbonds)
    d = len(psi.qsite)
    b = [len(q) for q in psi.qbonds]
    for i in range(len(b) - 1):
        shape = (b[i], d, b[i+1])
        if real:
            x = rng.normal(size=shape) / np.sqrt(b[i]*d*b[i+1])
        else:
            x = crandn(shape, rng) / np.sqrt(b[i]*d*b[i+1])
        enforce_qsparsity(x, [psi.qbonds[i], psi.qsite, -psi.qbonds[i+1]])
        psi.a[i] = x
    return psi


def local_orthonormalize_left_qr(a, a_next, qsite, qbonds):
    """QR of the left-grouped site tensor, R absorbed into the next site
    (mps.py:460-473)."""
    s = a.shape
    q0 = qnumber_flatten((qbonds[0], qsite))
    q, r, qbond = block_sparse_qr(a.reshape((s[0]*s[1], s[2])), q0, qbonds[1])
    a = q.reshape((s[0], s[1], q.shape[1]))
    a_next = np.tensordot(r, a_next, (1, 0))
    return a, a_next, qbond


def local_orthonormalize_right_qr(a, a_prev, qsite, qbonds):
    """QR of the right-grouped (transposed) site tensor, R absorbed into the
    previous site (mps.py:476-491)."""
    a = a.transpose((2, 1, 0))
    s = a.shape
    q0 = qnumber_flatten((-qbonds[1], qsite))
    q, r, qbond = block_sparse_qr(a.reshape((s[0]*s[1], s[2])), q0, -qbonds[0])
    a = q.reshape((s[0], s[1], q.shape[1])).transpose((2, 1, 0))
    a_prev = np.tensordot(a_prev, r, (2, 1))
    return a, a_prev, -qbond


def orthonormalize(psi, mode="left"):
    """Left or right QR orthonormalisation; returns the norm (mps.py:141-178)."""
    if len(psi.a) == 0:
        return 1
    if mode == "left":
        for i in range(len(psi.a) - 1):
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = local_orthonormalize_left_qr(
                psi.a[i], psi.a[i+1], psi.qsite, psi.qbonds[i:i+2])
        psi.a[-1], t, psi.qbonds[-1] = local_orthonormalize_left_qr(
            psi.a[-1], np.array([[[1]]]), psi.qsite, psi.qbonds[-2:])
        nrm = t[0, 0, 0].real
        if nrm < 0:
            psi.a[-1] = -psi.a[-1]
            nrm = -nrm
        return nrm
    if mode == "right":
        for i in reversed(range(1, len(psi.a))):
            psi.a[i], psi.a[i-1], psi.qbonds[i] = local_orthonormalize_right_qr(
                psi.a[i], psi.a[i-1], psi.qsite, psi.qbonds[i:i+2])
        psi.a[0], t, psi.qbonds[0] = local_orthonormalize_right_qr(
            psi.a[0], np.array([[[1]]]), psi.qsite, psi.qbonds[:2])
        nrm = t[0, 0, 0].real
        if nrm < 0:
            psi.a[0] = -psi.a[0]
            nrm = -nrm
        return nrm
    raise ValueError(f'`mode` = {mode} invalid; must be "left" or "right".')


def _merge_pair(a0, a1):
    """Merge neighbouring MPS tensors (mps.py:528-535)."""
    a = np.einsum(a0, (0, 1, 4), a1, (4, 2, 3), (0, 1, 2, 3), optimize=True)
    return a.reshape((a.shape[0], a.shape[1]*a.shape[2], a.shape[3]))


def mps_to_vector(psi):
    """Dense state vector (mps.py:292-301)."""
    v = psi.a[0]
    for x in psi.a[1:]:
        v = _merge_pair(v, x)
    assert v.shape[0] == 1 and v.shape[2] == 1
    return v.reshape(-1)


def _mpo_merge_pair(a0, a1):
    """Merge neighbouring MPO tensors: out[b0, (o0,o1), (i0,i1), b2]
    (mpo.py:314-322)."""
    a = np.einsum(a0, (0, 1, 3, 6), a1, (6, 2, 4, 5), (0, 1, 2, 3, 4, 5), optimize=True)
    s = a.shape
    return a.reshape((s[0], s[1]*s[2], s[3]*s[4], s[5]))


def mpo_to_matrix(op):
    """Dense operator matrix (mpo.py:225-235)."""
    m = op.a[0]
    for x in op.a[1:]:
        m = _mpo_merge_pair(m, x)
    assert m.shape[0] == 1 and m.shape[3] == 1
    return m.reshape((m.shape[1], m.shape[2]))


def _vdot_step_right(a, b, r):
    """One right step of the MPS inner product (mps.py:352-381)."""
    t = np.tensordot(a, r, 1)
    return np.tensordot(t, b.conj(), axes=((1, 2), (1, 2)))


def apply_mpo(op, psi):
    """MPO applied to an MPS (chain_ops.py:215-234): per site
    tensordot(W, A, (2, 1)) -> (chi_l, s, chi_r, D_l, D_r), transposed to
    (chi_l, D_l, s, chi_r, D_r) and grouped into (chi_l D_l, s, chi_r D_r); bond
    quantum numbers flattened pairwise (qnumber_flatten of (op, psi))."""
    assert np.array_equal(psi.qsite, op.qsite)
    assert psi.nsites == len(op.a)
    qbonds = [qnumber_flatten((op.qbonds[i], psi.qbonds[i])) for i in range(psi.nsites + 1)]
    out = OMPS(psi.qsite, qbonds)
    for i in range(psi.nsites):
        a = np.tensordot(op.a[i], psi.a[i], axes=(2, 1)).transpose((0, 3, 1, 2, 4))
        s = a.shape
        out.a[i] = a.reshape((s[0] * s[1], s[2], s[3] * s[4]))
        assert is_qsparse(out.a[i], (out.qbonds[i], out.qsite, -out.qbonds[i + 1]))
    return out


def mps_vdot(chi, psi):
    """<chi|psi> (mps.py:430-450)."""
    assert chi.nsites == psi.nsites
    if psi.nsites == 0:
        return 0
    t = np.identity(psi.a[-1].shape[2], dtype=psi.a[-1].dtype)
    for i in reversed(range(psi.nsites)):
        t = _vdot_step_right(psi.a[i], chi.a[i], t)
    return t[0, 0]


def mps_norm(psi):
    """(mps.py:453-457)"""
    return np.sqrt(mps_vdot(psi, psi).real)


# ---------------------------------------------------------------------------
# chain contractions -- pytenet/chain_ops.py
# ---------------------------------------------------------------------------

def env_step_right(a, b, w, r):
    """Right environment step (chain_ops.py:16-57): returns r_next[l_a, chi_l, l_b]."""
    t = np.tensordot(a, r, 1)
    t = np.tensordot(w, t, axes=((2, 3), (1, 2)))
    t = t.transpose((2, 0, 1, 3))
    return np.tensordot(t, b.conj(), axes=((2, 3), (1, 2)))


def env_step_left(a, b, w, l):
    """Left environment step (chain_ops.py:60-99): returns l_next[r_a, chi_r, r_b]."""
    t = np.tensordot(l, b.conj(), axes=(2, 0))
    t = np.tensordot(w, t, axes=((0, 1), (1, 2)))
    return np.tensordot(a, t, axes=((0, 1), (2, 0)))


def compute_right_operator_blocks(psi, op):
    """All right environments (chain_ops.py:102-113)."""
    n = psi.nsites
    assert n == len(op.a)
    blocks = [None] * n
    blocks[n-1] = np.array([[[1]]])
    for i in reversed(range(n - 1)):
        blocks[i] = env_step_right(psi.a[i+1], psi.a[i+1], op.a[i+1], blocks[i+1])
    return blocks


def apply_local_hamiltonian(a, w, l, r):
    """H_eff . A (chain_ops.py:237-279)."""
    t = np.tensordot(a, r, 1)
    t = np.tensordot(w, t, axes=((2, 3), (1, 2)))
    return np.tensordot(l, t, axes=((0, 1), (2, 0)))


def apply_local_bond_contraction(c, l, r):
    """Zero-site H_eff . C (chain_ops.py:282-317)."""
    t = np.tensordot(c, r, 1)
    return np.tensordot(l, t, axes=((0, 1), (0, 1)))


def mpo_inner_product(chi, op, psi):
    """<chi|op|psi> (chain_ops.py:165-189)."""
    if psi.nsites == 0:
        return 0
    n = psi.a[-1].shape[2]
    t = np.identity(n, dtype=psi.a[-1].dtype).reshape((n, 1, n))
    for i in reversed(range(psi.nsites)):
        t = env_step_right(psi.a[i], chi.a[i], op.a[i], t)
    assert t.shape == (1, 1, 1)
    return t[0, 0, 0]


def mpo_average(psi, op):
    """<psi|op|psi> (chain_ops.py:151-162)."""
    return mpo_inner_product(psi, op, psi)


# ---------------------------------------------------------------------------
# Krylov core -- pytenet/krylov.py
# ---------------------------------------------------------------------------

def lanczos_iteration(afunc, vstart, numiter):
    """Three-term Lanczos without re-orthogonalisation; early stop when
    beta < 100 n eps (krylov.py:12-57)."""
    vstart = np.asarray(vstart)
    nrmv = np.linalg.norm(vstart)
    assert nrmv > 0
    vstart = vstart / nrmv
    alpha = np.zeros(numiter)
    beta = np.zeros(numiter - 1)
    v = np.zeros((numiter, len(vstart)), dtype=vstart.dtype)
    v[0] = vstart
    for j in range(numiter - 1):
        w = afunc(v[j])
        alpha[j] = np.vdot(w, v[j]).real
        w -= alpha[j]*v[j] + (beta[j-1]*v[j-1] if j > 0 else 0)
        beta[j] = np.linalg.norm(w)
        if beta[j] < 100*len(vstart)*np.finfo(float).eps:
            warnings.warn(f"beta[{j}] ~= 0 encountered during Lanczos iteration.",
                          RuntimeWarning)
            m = j + 1
            return alpha[:m], beta[:m-1], v[:m, :].T
        v[j+1] = w / beta[j]
    j = numiter - 1
    w = afunc(v[j])
    alpha[j] = np.vdot(w, v[j]).real
    return alpha, beta, v.T


def eigh_tridiag(d, e):
    """Dense eigen-decomposition of the tridiagonal matrix (krylov.py:142-150)."""
    t = np.diag(d) + np.diag(e, k=1) + np.diag(e, k=-1)
    return np.linalg.eigh(t)


def expm_krylov(afunc, vec, dt, numiter):
    """Hermitian Krylov approximation of expm(dt A) vec (krylov.py:122-136)."""
    alpha, beta, v = lanczos_iteration(afunc, vec, numiter)
    w, u = eigh_tridiag(alpha, beta)
    return v @ (u @ (np.linalg.norm(vec) * np.exp(dt*w) * u[0]))


def eigh_krylov(afunc, vstart, numiter, numeig):
    """Lowest Ritz pairs (krylov.py:110-119)."""
    alpha, beta, v = lanczos_iteration(afunc, vstart, numiter)
    w, u = eigh_tridiag(alpha, beta)
    return w[:numeig], v @ u[:, :numeig]


# ---------------------------------------------------------------------------
# sweeps -- pytenet/tdvp.py, pytenet/dmrg.py
# ---------------------------------------------------------------------------

def _site_step(l, r, w, a, dt, numiter):
    """(tdvp.py:223-229)"""
    return expm_krylov(lambda x: apply_local_hamiltonian(x.reshape(a.shape), w, l, r).reshape(-1),
                       a.reshape(-1), -dt, numiter).reshape(a.shape)


def _bond_step(l, r, c, dt, numiter):
    """(tdvp.py:232-238)"""
    return expm_krylov(lambda x: apply_local_bond_contraction(x.reshape(c.shape), l, r).reshape(-1),
                       c.reshape(-1), -dt, numiter).reshape(c.shape)


def _check_rblocks(psi, op, rblocks):
    for i, rb in enumerate(rblocks):
        assert is_qsparse(rb, [psi.qbonds[i+1], op.qbonds[i+1], -psi.qbonds[i+1]]), \
            "sparsity pattern of operator blocks must match quantum numbers"


def tdvp_setup(op, psi):
    """The set-up of tdvp_singlesite (tdvp.py:45-63): right-normalise `psi`, build
    the right operator blocks. Returns (nrm, lblocks, rblocks)."""
    n = len(op.a)
    assert n == psi.nsites
    nrm = orthonormalize(psi, mode="right")
    rblocks = compute_right_operator_blocks(psi, op)
    lblocks = [None] * n
    lblocks[0] = np.array([[[1]]], dtype=rblocks[0].dtype)
    _check_rblocks(psi, op, rblocks)
    return nrm, lblocks, rblocks


def tdvp_step(op, psi, lblocks, rblocks, dt, numiter_lanczos):
    """One symmetric time step of tdvp_singlesite (the body of the loop at
    tdvp.py:65-115); `psi`, `lblocks` and `rblocks` are updated in place."""
    n = len(op.a)
    for i in range(n - 1):
        psi.a[i] = _site_step(lblocks[i], rblocks[i], op.a[i], psi.a[i], 0.5*dt,
                              numiter_lanczos)
        s = psi.a[i].shape
        q, c, psi.qbonds[i+1] = block_sparse_qr(
            psi.a[i].reshape((s[0]*s[1], s[2])),
            qnumber_flatten((psi.qbonds[i], psi.qsite)), psi.qbonds[i+1])
        psi.a[i] = q.reshape((s[0], s[1], q.shape[1]))
        lblocks[i+1] = env_step_left(psi.a[i], psi.a[i], op.a[i], lblocks[i])
        c = _bond_step(lblocks[i+1], rblocks[i], c, -0.5*dt, numiter_lanczos)
        psi.a[i+1] = np.tensordot(c, psi.a[i+1], (1, 0))
    i = n - 1
    psi.a[i] = _site_step(lblocks[i], rblocks[i], op.a[i], psi.a[i], dt, numiter_lanczos)
    for i in reversed(range(1, n)):
        psi.a[i] = psi.a[i].transpose((2, 1, 0))
        s = psi.a[i].shape
        q, c, qbond = block_sparse_qr(
            psi.a[i].reshape((s[0]*s[1], s[2])),
            qnumber_flatten((-psi.qbonds[i+1], psi.qsite)), -psi.qbonds[i])
        psi.qbonds[i] = -qbond
        psi.a[i] = q.reshape((s[0], s[1], q.shape[1])).transpose((2, 1, 0))
        rblocks[i-1] = env_step_right(psi.a[i], psi.a[i], op.a[i], rblocks[i])
        c = np.transpose(c)
        c = _bond_step(lblocks[i], rblocks[i-1], c, -0.5*dt, numiter_lanczos)
        psi.a[i-1] = np.tensordot(psi.a[i-1], c, (2, 0))
        psi.a[i-1] = _site_step(lblocks[i-1], rblocks[i-1], op.a[i-1], psi.a[i-1],
                                0.5*dt, numiter_lanczos)


def tdvp_singlesite(op, psi, dt, numsteps, numiter_lanczos=25):
    """Symmetric single-site TDVP; `psi` is overwritten; returns the initial
    norm (tdvp.py:26-118)."""
    nrm, lblocks, rblocks = tdvp_setup(op, psi)
    for _ in range(numsteps):
        tdvp_step(op, psi, lblocks, rblocks, dt, numiter_lanczos)
    return nrm


def _minimize_local_energy(w, l, r, a, numiter):
    """(dmrg.py:181-189)"""
    en, u = eigh_krylov(lambda x: apply_local_hamiltonian(x.reshape(a.shape), w, l, r).reshape(-1),
                        a.reshape(-1), numiter, 1)
    return en[0], u[:, 0].reshape(a.shape)


def dmrg_singlesite(op, psi, numsweeps, numiter_lanczos=25):
    """Single-site DMRG; `psi` is overwritten; returns the energy after each
    sweep (dmrg.py:22-93)."""
    n = len(op.a)
    assert n == psi.nsites
    orthonormalize(psi, mode="right")
    rblocks = compute_right_operator_blocks(psi, op)
    lblocks = [None] * n
    lblocks[0] = np.array([[[1]]], dtype=rblocks[0].dtype)
    _check_rblocks(psi, op, rblocks)
    en_min = np.zeros(numsweeps)
    for k in range(numsweeps):
        en = 0
        for i in range(n - 1):
            en, psi.a[i] = _minimize_local_energy(op.a[i], lblocks[i], rblocks[i], psi.a[i],
                                                  numiter_lanczos)
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = local_orthonormalize_left_qr(
                psi.a[i], psi.a[i+1], psi.qsite, psi.qbonds[i:i+2])
            lblocks[i+1] = env_step_left(psi.a[i], psi.a[i], op.a[i], lblocks[i])
        for i in reversed(range(1, n)):
            en, psi.a[i] = _minimize_local_energy(op.a[i], lblocks[i], rblocks[i], psi.a[i],
                                                  numiter_lanczos)
            psi.a[i], psi.a[i-1], psi.qbonds[i] = local_orthonormalize_right_qr(
                psi.a[i], psi.a[i-1], psi.qsite, psi.qbonds[i:i+2])
            rblocks[i-1] = env_step_right(psi.a[i], psi.a[i], op.a[i], rblocks[i])
        psi.a[0], _, psi.qbonds[0] = local_orthonormalize_right_qr(
            psi.a[0], np.array([[[1]]]), psi.qsite, psi.qbonds[:2])
        en_min[k] = en
    return en_min


# ---------------------------------------------------------------------------
# two-site sweeps (the next algorithm after the single-site path) --
# pytenet/bond_ops.py, pytenet/block_sparse_util.py, pytenet/mps.py,
# pytenet/tdvp.py:121-220, pytenet/dmrg.py:96-178
# ---------------------------------------------------------------------------

def retained_bond_indices(s, tol):
    """Singular values kept: those whose normalised squares, accumulated from the
    smallest up, exceed tol (bond_ops.py:23-38)."""
    w = np.linalg.norm(s)
    if w == 0:
        return np.array([], dtype=int)
    s = (s / w) ** 2
    order = np.argsort(s)
    s[order] = np.cumsum(s[order])
    return np.where(s > tol)[0]


def block_sparse_svd(a, q0, q1):
    """SVD per common quantum-number block (block_sparse_util.py:264-330); returns
    (u, s, v, q) with the intermediate quantum numbers q, rows / columns in the
    input order."""
    a = np.asarray(a)
    q0 = np.asarray(q0)
    q1 = np.asarray(q1)
    assert is_qsparse(a, [q0, -q1])
    qis = common_qnumbers(q0, q1)
    if len(qis) == 0:
        assert np.linalg.norm(a) == 0
        u = np.zeros((a.shape[0], 1), dtype=a.dtype)
        v = np.zeros((1, a.shape[1]), dtype=a.dtype)
        if a.shape[0] > 0:
            u[0, 0] = 1
        return u, np.zeros(1), v, q0[:1]
    a, (idx0, q0s), (idx1, q1s) = sort_by_qnumbers(a, q0, q1)
    kmax = min(a.shape)
    u = np.zeros((a.shape[0], kmax), dtype=a.dtype)
    v = np.zeros((kmax, a.shape[1]), dtype=a.dtype)
    s = np.zeros(kmax)
    q = np.zeros(kmax, dtype=q0s.dtype)
    k = 0
    for qn in qis:
        rs, cs = _qslice(qn, q0s), _qslice(qn, q1s)
        ub, sb, vb = np.linalg.svd(a[rs, cs], full_matrices=False)
        u[rs, k:k + len(sb)] = ub
        v[k:k + len(sb), cs] = vb
        s[k:k + len(sb)] = sb
        q[k:k + len(sb)] = qn
        k += len(sb)
    u, v, s, q = u[:, :k], v[:k, :], s[:k], q[:k]
    if np.any(idx0 - np.arange(len(idx0))):
        u = u[np.argsort(idx0), :]
    if np.any(idx1 - np.arange(len(idx1))):
        v = v[:, np.argsort(idx1)]
    return u, s, v, q


def split_block_sparse_matrix_svd(a, q0, q1, tol):
    """Block-sparse SVD truncated by retained_bond_indices (block_sparse_util.py:244-258)."""
    u, s, v, q = block_sparse_svd(a, q0, q1)
    idx = retained_bond_indices(s, tol)
    return u[:, idx], s[idx], v[idx, :], q[idx]


def mps_split_tensor_svd(a, qsite0, qsite1, qbonds_outer, svd_distr, tol=0):
    """Split a (b0, d0 d1, b2) tensor into (b0, d0, b1) and (b1, d1, b2) by the
    truncated block-sparse SVD, singular values to the left or right factor
    (mps.py:538-568)."""
    qsite0, qsite1 = np.asarray(qsite0), np.asarray(qsite1)
    d0, d1 = len(qsite0), len(qsite1)
    assert d0 * d1 == a.shape[1]
    s = (a.shape[0], d0, d1, a.shape[2])
    q0 = qnumber_flatten([qbonds_outer[0], qsite0])
    q1 = qnumber_flatten([-qsite1, qbonds_outer[1]])
    a0, sigma, a1, qbond = split_block_sparse_matrix_svd(a.reshape((s[0]*s[1], s[2]*s[3])),
                                                         q0, q1, tol)
    a0 = a0.reshape((s[0], s[1], len(sigma)))
    a1 = a1.reshape((len(sigma), s[2], s[3]))
    if svd_distr == "left":
        a0 = a0 * sigma
    elif svd_distr == "right":
        a1 = a1 * sigma[:, None, None]
    elif svd_distr == "sqrt":
        r = np.sqrt(sigma)
        a0 = a0 * r
        a1 = a1 * r[:, None, None]
    else:
        raise ValueError('`svd_distr` parameter must be "left", "right" or "sqrt".')
    return a0, a1, qbond


def tdvp_twosite(op, psi, dt, numsteps, numiter_lanczos=25, tol_split=0):
    """Symmetric two-site TDVP; `psi` is overwritten (bond dimensions may change);
    returns the initial norm (tdvp.py:121-220)."""
    n = len(op.a)
    assert n == psi.nsites and n >= 2
    nrm = orthonormalize(psi, mode="right")
    rblocks = compute_right_operator_blocks(psi, op)
    lblocks = [None] * n
    lblocks[0] = np.array([[[1]]], dtype=rblocks[0].dtype)
    _check_rblocks(psi, op, rblocks)
    h2 = [_mpo_merge_pair(op.a[i], op.a[i+1]) for i in range(n - 1)]
    for _ in range(numsteps):
        for i in range(n - 2):
            a = _site_step(lblocks[i], rblocks[i+1], h2[i], _merge_pair(psi.a[i], psi.a[i+1]),
                           0.5*dt, numiter_lanczos)
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = mps_split_tensor_svd(
                a, psi.qsite, psi.qsite, (psi.qbonds[i], psi.qbonds[i+2]), "right", tol=tol_split)
            lblocks[i+1] = env_step_left(psi.a[i], psi.a[i], op.a[i], lblocks[i])
            psi.a[i+1] = _site_step(lblocks[i+1], rblocks[i+1], op.a[i+1], psi.a[i+1],
                                    -0.5*dt, numiter_lanczos)
        i = n - 2
        a = _site_step(lblocks[i], rblocks[i+1], h2[i], _merge_pair(psi.a[i], psi.a[i+1]),
                       dt, numiter_lanczos)
        psi.a[i], psi.a[i+1], psi.qbonds[i+1] = mps_split_tensor_svd(
            a, psi.qsite, psi.qsite, [psi.qbonds[i], psi.qbonds[i+2]], "left", tol=tol_split)
        rblocks[i] = env_step_right(psi.a[i+1], psi.a[i+1], op.a[i+1], rblocks[i+1])
        for i in reversed(range(n - 2)):
            psi.a[i+1] = _site_step(lblocks[i+1], rblocks[i+1], op.a[i+1], psi.a[i+1],
                                    -0.5*dt, numiter_lanczos)
            a = _site_step(lblocks[i], rblocks[i+1], h2[i], _merge_pair(psi.a[i], psi.a[i+1]),
                           0.5*dt, numiter_lanczos)
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = mps_split_tensor_svd(
                a, psi.qsite, psi.qsite, [psi.qbonds[i], psi.qbonds[i+2]], "left", tol=tol_split)
            rblocks[i] = env_step_right(psi.a[i+1], psi.a[i+1], op.a[i+1], rblocks[i+1])
    return nrm


def dmrg_twosite(op, psi, numsweeps, numiter_lanczos=25, tol_split=0):
    """Two-site DMRG; `psi` is overwritten; returns the energy after each sweep
    (dmrg.py:96-178)."""
    n = len(op.a)
    assert n == psi.nsites
    orthonormalize(psi, mode="right")
    rblocks = compute_right_operator_blocks(psi, op)
    lblocks = [None] * n
    lblocks[0] = np.array([[[1]]], dtype=rblocks[0].dtype)
    _check_rblocks(psi, op, rblocks)
    en_min = np.zeros(numsweeps)
    h2 = [_mpo_merge_pair(op.a[i], op.a[i+1]) for i in range(n - 1)]
    for k in range(numsweeps):
        en = 0
        for i in range(n - 2):
            en, a = _minimize_local_energy(h2[i], lblocks[i], rblocks[i+1],
                                           _merge_pair(psi.a[i], psi.a[i+1]), numiter_lanczos)
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = mps_split_tensor_svd(
                a, psi.qsite, psi.qsite, [psi.qbonds[i], psi.qbonds[i+2]], "right", tol=tol_split)
            lblocks[i+1] = env_step_left(psi.a[i], psi.a[i], op.a[i], lblocks[i])
        for i in reversed(range(n - 1)):
            en, a = _minimize_local_energy(h2[i], lblocks[i], rblocks[i+1],
                                           _merge_pair(psi.a[i], psi.a[i+1]), numiter_lanczos)
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = mps_split_tensor_svd(
                a, psi.qsite, psi.qsite, [psi.qbonds[i], psi.qbonds[i+2]], "left", tol=tol_split)
            rblocks[i] = env_step_right(psi.a[i+1], psi.a[i+1], op.a[i+1], rblocks[i+1])
        psi.a[0], _, psi.qbonds[0] = local_orthonormalize_right_qr(
            psi.a[0], np.array([[[1]]]), psi.qsite, psi.qbonds[:2])
        en_min[k] = en
    return en_min


def local_orthonormalize_left_svd(a, a_next, qsite, qbonds, tol):
    """Left-orthonormalise `a` by the truncated block-sparse SVD and absorb
    sigma v into the next tensor (mps.py, mps_local_orthonormalize_left_svd)."""
    s = a.shape
    q0 = qnumber_flatten((qbonds[0], qsite))
    u, sigma, v, qbond = split_block_sparse_matrix_svd(a.reshape((s[0]*s[1], s[2])), q0,
                                                       qbonds[1], tol)
    return u.reshape((s[0], s[1], u.shape[1])), np.tensordot(sigma[:, None] * v, a_next, (1, 0)), qbond


def local_orthonormalize_right_svd(a, a_prev, qsite, qbonds, tol):
    """Right-orthonormalise `a` by the truncated block-sparse SVD and absorb
    u sigma into the previous tensor (mps.py, mps_local_orthonormalize_right_svd)."""
    s = a.shape
    q1 = qnumber_flatten([-np.asarray(qsite), qbonds[1]])
    u, sigma, v, qbond = split_block_sparse_matrix_svd(a.reshape((s[0], s[1]*s[2])), qbonds[0],
                                                       q1, tol)
    return v.reshape((v.shape[0], s[1], s[2])), np.tensordot(a_prev, u * sigma, (2, 0)), qbond


def compress_svd(psi, tol, direction="left"):
    """SVD compression and orthonormalisation of an MPS in place; returns the
    original norm and the scaling factor of the compression (mps.py:196-236)."""
    n = psi.nsites
    if direction == "left":
        nrm = orthonormalize(psi, mode="right")
        for i in range(n - 1):
            psi.a[i], psi.a[i+1], psi.qbonds[i+1] = local_orthonormalize_left_svd(
                psi.a[i], psi.a[i+1], psi.qsite, psi.qbonds[i:i+2], tol)
        psi.a[-1], t, psi.qbonds[-1] = local_orthonormalize_left_svd(
            psi.a[-1], np.array([[[1]]]), psi.qsite, psi.qbonds[-2:], tol)
        assert t.shape == (1, 1, 1)
        psi.a[-1] = psi.a[-1] * (t[0, 0, 0] / abs(t[0, 0, 0]))
        return nrm, abs(t[0, 0, 0])
    if direction == "right":
        nrm = orthonormalize(psi, mode="left")
        for i in reversed(range(1, n)):
            psi.a[i], psi.a[i-1], psi.qbonds[i] = local_orthonormalize_right_svd(
                psi.a[i], psi.a[i-1], psi.qsite, psi.qbonds[i:i+2], tol)
        psi.a[0], t, psi.qbonds[0] = local_orthonormalize_right_svd(
            psi.a[0], np.array([[[1]]]), psi.qsite, psi.qbonds[:2], tol)
        assert t.shape == (1, 1, 1)
        psi.a[0] = psi.a[0] * (t[0, 0, 0] / abs(t[0, 0, 0]))
        return nrm, abs(t[0, 0, 0])
    raise ValueError(f'`direction` = {direction} invalid; must be "left" or "right".')


# ---------------------------------------------------------------------------
# compression from local density matrices -- pytenet/mps.py:238-290 (McCulloch,
# J. Stat. Mech. (2007) P10014), with block_sparse_eigh from
# pytenet/block_sparse_util.py:183-241 and the left partial contractions of
# pytenet/mps.py:384-427
# ---------------------------------------------------------------------------

def block_sparse_eigh(a, q0):
    """Hermitian eigendecomposition per quantum-number block of `a` (rows and
    columns carry q0), block_sparse_util.py:183-241: the blocks in the iteration
    order of the Python set of q0, eigenvalues ascending inside a block (LAPACK
    heevd), rows of u in the input order. Returns (u, evals, q)."""
    a = np.asarray(a)
    q0 = np.asarray(q0)
    order = list(set(q0))                      # the reference iterates set(q0)
    a_s, (idx0, q0s), (_, q1s) = sort_by_qnumbers(a, q0, q0)
    n = a_s.shape[0]
    u = np.zeros((n, n), dtype=a.dtype)
    ev = np.zeros(n)
    q = np.zeros(n, dtype=q0.dtype)
    k = 0
    for qn in order:
        rs, cs = _qslice(qn, q0s), _qslice(qn, q1s)
        w, v = np.linalg.eigh(a_s[rs, cs])
        u[rs, k:k + len(w)] = v
        ev[k:k + len(w)] = w
        q[k:k + len(w)] = qn
        k += len(w)
    u, ev, q = u[:, :k], ev[:k], q[:k]
    if np.any(idx0 - np.arange(len(idx0))):
        u = u[np.argsort(idx0), :]
    return u, ev, q


def mps_left_blocks(psi):
    """Left partial contractions of <psi|psi> (mps.py:384-427): blocks[0] = [[1]],
    blocks[i+1][r, r'] = sum a_i[l, s, r] (blocks[i] conj(a_i))[l, s, r']."""
    blocks = [np.identity(1, dtype=psi.a[0].dtype)]
    for a in psi.a:
        t = np.tensordot(blocks[-1], a.conj(), axes=(1, 0))
        blocks.append(np.tensordot(a, t, axes=((0, 1), (0, 1))))
    return blocks


def compress_density(psi, tol):
    """Rounding compression from local density matrices, right to left, in place
    (mps.py:238-290); returns (original norm, scaling factor of the compression)."""
    n = len(psi.a)
    lb = mps_left_blocks(psi)
    assert lb[-1].shape == (1, 1) and lb[-1][0, 0].real > 0
    nrm = np.sqrt(lb[-1][0, 0].real)
    b = np.array([[[1]]], dtype=psi.a[-1].dtype)
    u = np.array([[[1]]], dtype=psi.a[-1].dtype)
    for i in reversed(range(1, n)):
        b = np.tensordot(b, u.conj(), axes=((1, 2), (1, 2)))
        b = np.tensordot(psi.a[i], b, axes=((2,), (0,)))
        rho = np.tensordot(b, lb[i], axes=((0,), (0,)))
        rho = np.tensordot(rho, b.conj(), axes=((2,), (0,)))
        shp = rho.shape[:2]
        rho = rho.reshape((shp[0] * shp[1], -1))
        qr = qnumber_flatten((psi.qsite, -np.asarray(psi.qbonds[i + 1])))
        assert is_qsparse(rho, (qr, -qr))
        u, ev, qe = block_sparse_eigh(rho, qr)
        idx = retained_bond_indices(np.abs(ev), tol)   # eigenvalues can be slightly negative
        u = u[:, idx]
        qe = -qe[idx]
        u = u.reshape(shp[0], shp[1], u.shape[1]).transpose((2, 0, 1))
        psi.a[i] = u
        psi.qbonds[i] = qe
    b = np.tensordot(b, u.conj(), axes=((1, 2), (1, 2)))
    b = np.tensordot(psi.a[0], b, axes=((2,), (0,)))
    s = np.linalg.norm(b.reshape(-1))
    psi.a[0] = b / s
    return nrm, s / nrm
