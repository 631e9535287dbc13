"""
MPS compression on the GPU: MPS.compress(tol, "svd", direction) of the reference
(pytenet/mps.py:180-236, with mps_local_orthonormalize_left_svd / _right_svd) and
MPS.compress(tol, "density") (pytenet/mps.py:238-290, rounding by local density
matrices).

Each step splits one site tensor with the block-sparse SVD on the device
(ptn_svd per quantum-number block), keeps the singular values that the
reference's truncation rule keeps (decided on the host, exact), and absorbs
sigma V (or U sigma) into the neighbouring tensor with one GEMM. Singular vectors
carry a phase per value that need not equal LAPACK's, so site tensors can differ
from the reference's by such phases on the bonds; the state, the bond dimensions,
their quantum numbers, the norm and the compression factor do not.
"""

import numpy as np
import torch

from . import _lib
from .block_sparse import RowMajor, svd_execute, take_singular, _svd_scratch
from .bond_ops import retained_bond_indices
from .device import Workspace, call, device, empty, lib, ptr, stream_ptr, to_dev, to_host
from .qnumber import is_qsparse, qnumber_flatten, qr_plan

__all__ = ["compress_svd", "compress_density"]


def _split(x, rows, cols, q0, q1, tol):
    """Truncated block-sparse SVD of the device matrix x (rows x cols, row-major):
    u (rows x k), s (k, host and device), vh (k x cols), q (k,)."""
    plan = qr_plan(q0, q1)
    u, s, vh = svd_execute(plan, x, RowMajor(cols), _svd_scratch())
    s_host = s.cpu().numpy()
    idx = retained_bond_indices(s_host, tol)
    u, vh = take_singular(u, vh, idx)
    sk = s_host[idx]
    return u, sk, torch.from_numpy(np.ascontiguousarray(sk)).to(device()), vh, plan.qinterm[idx].copy()


def _gemm(M, N, K, a, b, out, ws, opa="N", opb="N"):
    """out (M x N) = op(a) op(b) on the FP64 tensor cores; a is stored M x K for
    "N" / "C" and K x M for "T" / "H", b likewise (row-major)."""
    L = lib()
    wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
    w = ws.get(wsb)
    lda = K if opa in "NC" else M
    ldb = N if opb in "NC" else K
    call(L.ptn_zgemm, opa.encode(), opb.encode(), M, N, K, _lib.cval(1), ptr(a), lda, 0, ptr(b),
         ldb, 0, _lib.cval(0), ptr(out), N, 0, 1, ptr(w), wsb, stream_ptr())


def compress_svd(psi, tol, direction="left"):
    """Compress and orthonormalise `psi` in place by site-local SVDs and singular
    value truncation; returns (original norm, scaling factor of the compression)
    (pytenet/mps.py:196-236)."""
    if direction not in ("left", "right"):
        raise ValueError(f'`direction` = {direction} invalid; must be "left" or "right".')
    L, st = lib(), stream_ptr()
    n = len(psi.a)
    nrm = psi.orthonormalize(mode="right" if direction == "left" else "left")
    qsite = np.asarray(psi.qsite)
    d = len(qsite)
    a = [to_dev(x) for x in psi.a]
    qb = [np.asarray(q).copy() for q in psi.qbonds]
    ws = Workspace()
    if direction == "left":
        for i in range(n):
            Dl, _, Dr = a[i].shape
            q0 = qnumber_flatten((qb[i], qsite))
            u, sk, skd, vh, q = _split(a[i], Dl * d, Dr, q0, qb[i + 1], tol)
            k = len(sk)
            if k > 0:
                call(L.ptn_diag_scale, ptr(vh), k, Dr, Dr, ptr(skd), 1, st)
            a[i] = u.view(Dl, d, k)
            qb[i + 1] = q
            if i + 1 < n:
                _, d1, Dr1 = a[i + 1].shape
                out = empty((k, d1, Dr1))
                _gemm(k, d1 * Dr1, Dr, vh, a[i + 1], out, ws)
                a[i + 1] = out
                assert is_qsparse(to_host(a[i]), [qb[i], qsite, -qb[i + 1]]), \
                    "sparsity pattern of MPS tensor does not match quantum numbers"
            else:
                # the last factor sigma V is 1 x 1: its phase goes into the last tensor
                t = complex(to_host(vh).reshape(-1)[0])
                call(L.ptn_scale, ptr(a[i]), ptr(a[i]), a[i].numel(), _lib.cval(t / abs(t)), st)
                scale = abs(t)
    else:
        for i in reversed(range(n)):
            Dl, _, Dr = a[i].shape
            q1 = qnumber_flatten((-qsite, qb[i + 1]))
            u, sk, skd, vh, q = _split(a[i], Dl, d * Dr, qb[i], q1, tol)
            k = len(sk)
            if k > 0:
                call(L.ptn_diag_scale, ptr(u), Dl, k, k, ptr(skd), 0, st)
            a[i] = vh.view(k, d, Dr)
            qb[i] = q
            if i > 0:
                Dl0, d0, _ = a[i - 1].shape
                out = empty((Dl0, d0, k))
                _gemm(Dl0 * d0, k, Dl, a[i - 1], u, out, ws)
                a[i - 1] = out
                assert is_qsparse(to_host(a[i]), [qb[i], qsite, -qb[i + 1]]), \
                    "sparsity pattern of MPS tensor does not match quantum numbers"
            else:
                t = complex(to_host(u).reshape(-1)[0])
                call(L.ptn_scale, ptr(a[i]), ptr(a[i]), a[i].numel(), _lib.cval(t / abs(t)), st)
                scale = abs(t)
    psi.a = [to_host(x).copy() for x in a]
    psi.qbonds = qb
    return nrm, scale


def _eigh_order(plan, qr):
    """Column order of block_sparse_eigh (pytenet/block_sparse_util.py:183-241) in
    terms of the block SVD's columns: blocks in the iteration order of the Python
    set of the row quantum numbers, each block's values ascending (the SVD gives
    them descending per block, in sorted quantum-number order)."""
    start = {}
    for rows, cols, k0, kb in plan.blocks:
        start[int(plan.qinterm[k0])] = (k0, kb)
    perm = []
    for qn in set(np.asarray(qr)):
        k0, kb = start[int(qn)]
        perm.extend(range(k0 + kb - 1, k0 - 1, -1))
    return np.asarray(perm, dtype=np.int64)


def compress_density(psi, tol):
    """Rounding compression from local density matrices, right to left, in place
    (pytenet/mps.py:238-290, McCulloch, J. Stat. Mech. (2007) P10014); returns
    (original norm, scaling factor of the compression).

    Every contraction is an FP64 GEMM on the device. The density matrix of a site,
    rho = B L B^H, is Hermitian positive semidefinite, so its eigenvectors per
    quantum-number block are the singular vectors of the device block SVD and
    |eigenvalue| = singular value; the columns are put in the reference's block
    and eigenvalue order (block_sparse_eigh), and the reference's truncation rule
    on |eigenvalues| decides which are kept (host, exact integers): bond dimensions
    and their quantum numbers agree with the reference's exactly, the tensors up to
    a phase per kept vector, the state as a whole to rounding."""
    L, st = lib(), stream_ptr()
    n = len(psi.a)
    qsite = np.asarray(psi.qsite)
    d = len(qsite)
    a = [to_dev(x) for x in psi.a]
    qb = [np.asarray(q).copy() for q in psi.qbonds]
    ws = Workspace()
    # left partial contractions of <psi|psi> (pytenet/mps.py:384-427)
    lb = [torch.ones((1, 1), dtype=torch.complex128, device=device())]
    for i in range(n):
        Dl, _, Dr = a[i].shape
        t = empty((Dl, d * Dr))
        _gemm(Dl, d * Dr, Dl, lb[i], a[i], t, ws, "N", "C")
        nxt = empty((Dr, Dr))
        _gemm(Dr, Dr, Dl * d, a[i], t, nxt, ws, "T", "N")
        lb.append(nxt)
    last = complex(to_host(lb[n]).reshape(-1)[0])
    assert lb[n].shape == (1, 1) and last.real > 0
    nrm = float(np.sqrt(last.real))
    b = torch.ones((1, 1, 1), dtype=torch.complex128, device=device())
    u = torch.ones((1, 1, 1), dtype=torch.complex128, device=device())
    for i in reversed(range(1, n)):
        B0, Ku = b.shape[0], u.shape[0]
        b2 = empty((B0, Ku))
        _gemm(B0, Ku, b.shape[1] * b.shape[2], b, u, b2, ws, "N", "H")
        Dl, _, Dr = a[i].shape
        b3 = empty((Dl, d, Ku))
        _gemm(Dl * d, Ku, Dr, a[i], b2, b3, ws)
        rho1 = empty((d * Ku, Dl))
        _gemm(d * Ku, Dl, Dl, b3, lb[i], rho1, ws, "T", "N")
        rho = empty((d * Ku, d * Ku))
        _gemm(d * Ku, d * Ku, Dl, rho1, b3, rho, ws, "N", "C")
        qr = qnumber_flatten((qsite, -qb[i + 1]))
        plan = qr_plan(qr, qr)
        uu, s, vh = svd_execute(plan, rho, RowMajor(d * Ku), _svd_scratch())
        perm = _eigh_order(plan, qr)
        ev = s.cpu().numpy()[perm]
        idx = retained_bond_indices(ev, tol)
        keep = perm[idx]
        k = len(keep)
        uk, _ = take_singular(uu, vh, keep)
        # u (d Ku x k) -> site tensor (k, d, Ku)
        site = empty((k, d, Ku))
        call(L.ptn_transpose_210, ptr(uk), ptr(site), d * Ku, 1, k, st)
        a[i] = site
        qb[i] = -plan.qinterm[keep]
        u, b = site, b3
    B0, Ku = b.shape[0], u.shape[0]
    b2 = empty((B0, Ku))
    _gemm(B0, Ku, b.shape[1] * b.shape[2], b, u, b2, ws, "N", "H")
    Dl, _, Dr = a[0].shape
    b3 = empty((Dl, d, Ku))
    _gemm(Dl * d, Ku, Dr, a[0], b2, b3, ws)
    s0 = float(torch.linalg.vector_norm(b3).item())
    call(L.ptn_scale, ptr(b3), ptr(b3), b3.numel(), _lib.cval(1.0 / s0), st)
    a[0] = b3
    psi.a = [to_host(x).copy() for x in a]
    psi.qbonds = qb
    return nrm, s0 / nrm
