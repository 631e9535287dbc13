"""
MPS compression by site-local truncated SVDs on the GPU: MPS.compress(tol, "svd",
direction) of the reference (pytenet/mps.py:180-236, with
mps_local_orthonormalize_left_svd / _right_svd).

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

__all__ = ["compress_svd"]


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


def _gemm(M, N, K, a, b, out, ws):
    L = lib()
    wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
    w = ws.get(wsb)
    call(L.ptn_zgemm, b"N", b"N", M, N, K, _lib.cval(1), ptr(a), K, 0, ptr(b), N, 0,
         _lib.cval(0), ptr(out), N, 0, 1, ptr(w), wsb, stream_ptr())


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
