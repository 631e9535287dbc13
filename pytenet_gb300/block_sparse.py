"""
Block-sparse QR and SVD on the device: block_sparse_qr and block_sparse_svd of
pytenet/block_sparse_util.py:106-180 and :244-330.

The integer plan (qnumber.QRPlan) says which rows / columns form each quantum-
number block; the device gathers each block into a dense matrix, runs the
Householder QR kernel, and scatters Q and R straight into their final layouts.
Any transposition of the sweep (the right-to-left step factors the (2,1,0)
transpose of the site tensor, pytenet/tdvp.py:95-104) is folded into the gather /
scatter index maps, so nothing is transposed separately in the block path.
"""

import numpy as np
import torch

from . import _lib
from .device import call, empty, lib, ptr, stream_ptr, to_dev, to_host, Workspace
from .qnumber import qr_plan, is_qsparse

__all__ = ["RowMajor", "ColMajor", "Flip3", "qr_execute", "block_sparse_qr", "svd_execute",
           "block_sparse_svd", "split_block_sparse_matrix_svd"]


class RowMajor:
    """Matrix element (r, c) at r*ld + c."""

    def __init__(self, ld):
        self.ld = int(ld)

    def offsets(self, rows, cols):
        return np.asarray(rows, np.int64) * self.ld, np.asarray(cols, np.int64)

    def key(self):
        return ("R", self.ld)


class ColMajor:
    """Matrix element (r, c) at c*ld + r (a transposed row-major matrix)."""

    def __init__(self, ld):
        self.ld = int(ld)

    def offsets(self, rows, cols):
        return np.asarray(rows, np.int64), np.asarray(cols, np.int64) * self.ld

    def key(self):
        return ("C", self.ld)


class Flip3:
    """Tensor t of shape (X, d, Y) seen as the matrix t.transpose((2,1,0)).reshape(Y*d, X):
    element (y*d + s, x) at x*d*Y + s*Y + y."""

    def __init__(self, d, Y):
        self.d, self.Y = int(d), int(Y)

    def offsets(self, rows, cols):
        rows = np.asarray(rows, np.int64)
        y, s = rows // self.d, rows % self.d
        return s * self.Y + y, np.asarray(cols, np.int64) * (self.d * self.Y)

    def key(self):
        return ("F", self.d, self.Y)


def _dev_i64(x):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.int64)).to("cuda")


def _block_maps(plan, src_view, q_view, r_view):
    """Device offset arrays per block, cached on the plan."""
    key = (src_view.key(), q_view.key(), r_view.key())
    maps = plan.dev_cache.get(key)
    if maps is None:
        maps = []
        for rows, cols, k0, kb in plan.blocks:
            kk = np.arange(k0, k0 + kb, dtype=np.int64)
            sro, sco = src_view.offsets(rows, cols)
            qro, qco = q_view.offsets(rows, kk)
            rro, rco = r_view.offsets(kk, cols)
            maps.append(tuple(_dev_i64(x) for x in (sro, sco, qro, qco, rro, rco)))
        plan.dev_cache[key] = maps
    return maps


class QRScratch:
    """Device scratch of the block QR (grow-only)."""

    def __init__(self):
        self.ws = Workspace()
        self.work = Workspace()
        self.qb = Workspace()
        self.rb = Workspace()


def qr_execute(plan, src, src_view, q_dst, q_view, r_dst, r_view, scratch):
    """Run the planned block QR. `src` is a device complex128 tensor (any shape,
    read through src_view); Q (m x K) and R (K x n) are written through q_view /
    r_view into q_dst / r_dst, which are zeroed first. `src` must not alias the
    destinations."""
    L = lib()
    st = stream_ptr()
    q_dst.zero_()
    r_dst.zero_()
    if plan.empty:
        qro, qco = q_view.offsets([0], [0])
        q_dst.view(-1)[int(qro[0] + qco[0])] = 1.0
        return
    for (rows, cols, k0, kb), (sro, sco, qro, qco, rro, rco) in zip(
            plan.blocks, _block_maps(plan, src_view, q_view, r_view)):
        mb, nb = len(rows), len(cols)
        work = scratch.work.get(mb * nb * 16)
        qb = scratch.qb.get(mb * kb * 16)
        rb = scratch.rb.get(kb * nb * 16)
        wsb = L.ptn_qr_workspace_bytes(mb, nb)
        ws = scratch.ws.get(wsb)
        call(L.ptn_gather, ptr(src), ptr(sro), ptr(sco), mb, nb, ptr(work), st)
        call(L.ptn_qr, ptr(work), mb, nb, ptr(qb), kb, ptr(rb), nb, ptr(ws), wsb, st)
        call(L.ptn_scatter, ptr(qb), kb, ptr(qro), ptr(qco), mb, kb, ptr(q_dst), st)
        call(L.ptn_scatter, ptr(rb), nb, ptr(rro), ptr(rco), kb, nb, ptr(r_dst), st)


_SCRATCH = None


def block_sparse_qr(a, q0, q1):
    """Drop-in for pytenet.block_sparse_qr: block-wise reduced QR of `a`
    respecting quantum numbers; returns (q, r, qinterm). `a` may be a NumPy array
    (results come back as NumPy arrays) or a complex128 CUDA tensor."""
    global _SCRATCH
    host = not isinstance(a, torch.Tensor)
    assert a.ndim == 2
    assert len(q0) == a.shape[0] and len(q1) == a.shape[1]
    q0 = np.asarray(q0)
    q1 = np.asarray(q1)
    assert is_qsparse(a, [q0, -q1])
    plan = qr_plan(q0, q1)
    m, n = a.shape
    src = to_dev(a)
    if plan.empty:
        assert float(torch.linalg.vector_norm(src).item()) == 0.0
    q = empty((m, plan.K))
    r = empty((plan.K, n))
    if _SCRATCH is None:
        _SCRATCH = QRScratch()
    qr_execute(plan, src, RowMajor(n), q, RowMajor(plan.K), r, RowMajor(n), _SCRATCH)
    if host:
        return to_host(q), to_host(r), plan.qinterm.copy()
    return q, r, plan.qinterm.copy()


# --------------------------------------------------------------------------- SVD

class SVDScratch:
    """Device scratch of the block SVD (grow-only)."""

    def __init__(self):
        self.ws = Workspace()
        self.work = Workspace()
        self.ub = Workspace()
        self.vb = Workspace()


def svd_execute(plan, src, src_view, scratch):
    """Block SVD on the device following a QRPlan (its blocks are the SVD's: rows and
    columns of one common quantum number, min(rows, cols) singular values each, in
    the plan's quantum-number order). Returns device tensors u (m x K), s (K,),
    vh (K x n) with rows / columns in the input order (block_sparse_util.py:264-330)."""
    L = lib()
    st = stream_ptr()
    m, n = plan.m, plan.n
    u = empty((m, plan.K))
    vh = empty((plan.K, n))
    s = torch.zeros(plan.K, dtype=torch.float64, device="cuda")
    u.zero_()
    vh.zero_()
    if plan.empty:
        # no common quantum number: u = e_0, s = 0, vh = 0 (block_sparse_util.py:282-289)
        if m > 0:
            u.view(-1)[0] = 1.0
        return u, s, vh
    uv, vv = RowMajor(plan.K), RowMajor(n)
    for (rows, cols, k0, kb), (sro, sco, uro, uco, vro, vco) in zip(
            plan.blocks, _block_maps(plan, src_view, uv, vv)):
        mb, nb = len(rows), len(cols)
        work = scratch.work.get(mb * nb * 16)
        ub = scratch.ub.get(mb * kb * 16)
        vb = scratch.vb.get(kb * nb * 16)
        wsb = L.ptn_svd_workspace_bytes(mb, nb)
        ws = scratch.ws.get(wsb)
        call(L.ptn_gather, ptr(src), ptr(sro), ptr(sco), mb, nb, ptr(work), st)
        call(L.ptn_svd, ptr(work), mb, nb, nb, ptr(ub), kb, ptr(s[k0:k0 + kb]), ptr(vb), nb, None,
             ptr(ws), wsb, st)
        call(L.ptn_scatter, ptr(ub), kb, ptr(uro), ptr(uco), mb, kb, ptr(u), st)
        call(L.ptn_scatter, ptr(vb), nb, ptr(vro), ptr(vco), kb, nb, ptr(vh), st)
    return u, s, vh


_SVD_SCRATCH = None


def _svd_scratch():
    global _SVD_SCRATCH
    if _SVD_SCRATCH is None:
        _SVD_SCRATCH = SVDScratch()
    return _SVD_SCRATCH


def block_sparse_svd(a, q0, q1):
    """Drop-in for pytenet.block_sparse_svd (pytenet/block_sparse_util.py:244-330):
    SVD per common quantum-number block; returns (u, s, v, q). NumPy input gives
    NumPy results, a complex128 CUDA tensor gives device tensors (q stays on the
    host). Singular vectors may differ from LAPACK's by a phase per value."""
    host = not isinstance(a, torch.Tensor)
    assert a.ndim == 2
    q0 = np.asarray(q0)
    q1 = np.asarray(q1)
    assert len(q0) == a.shape[0] and len(q1) == a.shape[1]
    assert is_qsparse(a, [q0, -q1])
    plan = qr_plan(q0, q1)
    src = to_dev(a)
    if plan.empty:
        assert float(torch.linalg.vector_norm(src).item()) == 0.0
    u, s, vh = svd_execute(plan, src, RowMajor(a.shape[1]), _svd_scratch())
    q = plan.qinterm.copy()
    if host:
        return to_host(u), s.cpu().numpy(), to_host(vh), q
    return u, s, vh, q


def split_block_sparse_matrix_svd(a, q0, q1, tol):
    """Drop-in for pytenet.split_block_sparse_matrix_svd (pytenet/bond_ops.py:41-53):
    block-sparse SVD truncated by retained_bond_indices. The truncation is decided
    on the host from the singular values (integer bookkeeping, exact); the
    retained columns / rows are gathered on the device."""
    from .bond_ops import retained_bond_indices
    host = not isinstance(a, torch.Tensor)
    u, s, vh, q = block_sparse_svd(to_dev(a) if host else a, q0, q1)
    s_host = s.cpu().numpy()
    idx = retained_bond_indices(s_host, tol)
    u, vh = take_singular(u, vh, idx)
    s_keep = s_host[idx]
    q = q[idx]
    if host:
        return to_host(u), s_keep, to_host(vh), q
    return u, torch.from_numpy(np.ascontiguousarray(s_keep)).to(u.device), vh, q


def take_singular(u, vh, idx):
    """u[:, idx] and vh[idx, :], gathered on the device."""
    L = lib()
    st = stream_ptr()
    m, K = u.shape
    n = vh.shape[1]
    k = len(idx)
    ut = empty((m, k))
    vt = empty((k, n))
    if k > 0:
        # the offset arrays stay referenced until the gathers are enqueued: a freed
        # temporary could be handed to the next upload before the kernel reads it
        idx64 = np.asarray(idx, np.int64)
        u_rows = _dev_i64(np.arange(m, dtype=np.int64) * K)
        u_cols = _dev_i64(idx64)
        v_rows = _dev_i64(idx64 * n)
        v_cols = _dev_i64(np.arange(n, dtype=np.int64))
        call(L.ptn_gather, ptr(u), ptr(u_rows), ptr(u_cols), m, k, ptr(ut), st)
        call(L.ptn_gather, ptr(vh), ptr(v_rows), ptr(v_cols), k, n, ptr(vt), st)
    return ut, vt
