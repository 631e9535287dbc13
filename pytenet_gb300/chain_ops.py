"""
Chain contractions with the signatures of pytenet/chain_ops.py, computed by the
GPU kernels. Inputs may be NumPy arrays (results are returned as NumPy arrays,
like the reference) or complex128 CUDA tensors (results stay on the device).
"""

import numpy as np
import torch

from . import _lib
from .device import Workspace, call, device, empty, lib, ptr, stream_ptr, to_dev, to_host

__all__ = ["apply_local_hamiltonian", "apply_local_bond_contraction",
           "contraction_operator_step_left", "contraction_operator_step_right",
           "compute_right_operator_blocks", "mpo_average", "mpo_inner_product",
           "mps_vdot", "mps_norm"]

_WS = Workspace()


def _is_host(*xs):
    return not any(isinstance(x, torch.Tensor) for x in xs)


def _ret(t, host):
    return to_host(t) if host else t


def apply_local_hamiltonian(a, w, l, r, precision="fp64"):
    """H_eff . a (pytenet/chain_ops.py:237-279): out[l2, s, r2]."""
    from .engine import prec_code
    assert a.ndim == 3 and w.ndim == 4 and l.ndim == 3 and r.ndim == 3
    host = _is_host(a, w, l, r)
    Dl, d, Dr = a.shape
    cl, cr = w.shape[0], w.shape[3]
    assert tuple(l.shape) == (Dl, cl, Dl) and tuple(r.shape) == (Dr, cr, Dr)
    assert w.shape[1] == d and w.shape[2] == d
    A, W, Lt, R = (to_dev(x) for x in (a, w, l, r))
    out = empty((Dl, d, Dr))
    p = prec_code(precision)
    L = lib()
    wsb = L.ptn_heff_workspace_bytes(Dl, d, Dr, cl, cr, p)
    call(L.ptn_heff_apply, ptr(A), ptr(W), ptr(Lt), ptr(R), ptr(out), Dl, d, Dr, cl, cr, p,
         ptr(_WS.get(wsb)), wsb, stream_ptr())
    return _ret(out, host)


def apply_local_bond_contraction(c, l, r, precision="fp64"):
    """Zero-site H_eff . c (pytenet/chain_ops.py:282-317): out[l2, r2]."""
    from .engine import prec_code
    assert c.ndim == 2 and l.ndim == 3 and r.ndim == 3
    host = _is_host(c, l, r)
    Dl, Dr = c.shape
    chi = l.shape[1]
    assert tuple(l.shape) == (Dl, chi, Dl) and tuple(r.shape) == (Dr, chi, Dr)
    Cm, Lt, R = (to_dev(x) for x in (c, l, r))
    out = empty((Dl, Dr))
    p = prec_code(precision)
    L = lib()
    wsb = L.ptn_bond_workspace_bytes(Dl, Dr, chi, p)
    call(L.ptn_bond_apply, ptr(Cm), ptr(Lt), ptr(R), ptr(out), Dl, Dr, chi, p, ptr(_WS.get(wsb)),
         wsb, stream_ptr())
    return _ret(out, host)


def contraction_operator_step_left(a, b, w, l, precision="fp64"):
    """Left environment step (pytenet/chain_ops.py:60-99): l_next[r_a, chi_r, r_b]."""
    from .engine import prec_code
    p = prec_code(precision)
    assert a.ndim == 3 and b.ndim == 3 and w.ndim == 4 and l.ndim == 3
    assert tuple(a.shape) == tuple(b.shape), "a and b must have equal shapes"
    host = _is_host(a, b, w, l)
    Dl, d, Dr = a.shape
    cl, cr = w.shape[0], w.shape[3]
    assert tuple(l.shape) == (Dl, cl, Dl)
    A, B, W, Lt = (to_dev(x) for x in (a, b, w, l))
    out = empty((Dr, cr, Dr))
    L = lib()
    wsb = L.ptn_env_workspace_bytes(Dl, d, Dr, cl, cr, p)
    call(L.ptn_env_step_left, ptr(A), ptr(B), ptr(W), ptr(Lt), ptr(out), Dl, d, Dr, cl, cr, p,
         ptr(_WS.get(wsb)), wsb, stream_ptr())
    return _ret(out, host)


def contraction_operator_step_right(a, b, w, r, precision="fp64"):
    """Right environment step (pytenet/chain_ops.py:16-57): r_next[l_a, chi_l, l_b]."""
    from .engine import prec_code
    p = prec_code(precision)
    assert a.ndim == 3 and b.ndim == 3 and w.ndim == 4 and r.ndim == 3
    assert tuple(a.shape) == tuple(b.shape), "a and b must have equal shapes"
    host = _is_host(a, b, w, r)
    Dl, d, Dr = a.shape
    cl, cr = w.shape[0], w.shape[3]
    assert tuple(r.shape) == (Dr, cr, Dr)
    A, B, W, R = (to_dev(x) for x in (a, b, w, r))
    out = empty((Dl, cl, Dl))
    L = lib()
    wsb = L.ptn_env_workspace_bytes(Dl, d, Dr, cl, cr, p)
    call(L.ptn_env_step_right, ptr(A), ptr(B), ptr(W), ptr(R), ptr(out), Dl, d, Dr, cl, cr, p,
         ptr(_WS.get(wsb)), wsb, stream_ptr())
    return _ret(out, host)


def compute_right_operator_blocks(psi, op):
    """All right environments (pytenet/chain_ops.py:102-113), as device tensors."""
    n = psi.nsites
    assert n == op.nsites
    blocks = [None] * n
    blocks[n - 1] = to_dev(np.array([[[1.0]]]))
    for i in reversed(range(n - 1)):
        blocks[i] = contraction_operator_step_right(to_dev(psi.a[i + 1]), to_dev(psi.a[i + 1]),
                                                    to_dev(op.a[i + 1]), blocks[i + 1])
    return blocks


def _tensors(x):
    """Site tensors of an MPS / MPO (host arrays, uploaded per use) or a list of
    device tensors (a device-resident run's sites: no host round trip)."""
    return x.a if hasattr(x, "a") else list(x)


def mpo_inner_product(chi, op, psi):
    """<chi|op|psi> (pytenet/chain_ops.py:165-189); chi and psi must share their
    bond dimensions (the square-environment kernels). Each argument is an MPS /
    MPO or a list of device site tensors."""
    A, B, W = _tensors(psi), _tensors(chi), _tensors(op)
    assert len(A) == len(B) == len(W)
    if len(A) == 0:
        return 0
    n = A[-1].shape[2]
    t = to_dev(np.identity(n).reshape((n, 1, n)))
    for i in reversed(range(len(A))):
        t = contraction_operator_step_right(to_dev(A[i]), to_dev(B[i]), to_dev(W[i]), t)
    assert tuple(t.shape) == (1, 1, 1)
    return complex(t.reshape(-1)[0].item())


def mpo_average(psi, op):
    """<psi|op|psi> (pytenet/chain_ops.py:151-162)."""
    return mpo_inner_product(psi, op, psi)


def _zgemm(opa, opb, M, N, K, A, lda, B, ldb, Cout, ldc):
    L = lib()
    wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
    call(L.ptn_zgemm, opa, opb, M, N, K, _lib.cval(1), ptr(A), lda, 0, ptr(B), ldb, 0,
         _lib.cval(0), ptr(Cout), ldc, 0, 1, ptr(_WS.get(wsb)), wsb, stream_ptr())


def mps_vdot(chi, psi):
    """<chi|psi> (pytenet/mps.py:430-450), contracted from the right on the GPU;
    chi and psi are MPS or lists of device site tensors."""
    A, B = _tensors(psi), _tensors(chi)
    assert len(A) == len(B)
    if len(A) == 0:
        return 0
    n = A[-1].shape[2]
    t = to_dev(np.identity(n))               # (Dpsi_r, Dchi_r)
    for i in reversed(range(len(A))):
        a = to_dev(A[i])
        b = to_dev(B[i])
        Dl, d, Dr = a.shape
        El, _, Er = b.shape
        # u[(l, s), e] = sum_r a[(l, s), r] t[r, e]
        u = empty((Dl, d, Er))
        _zgemm(b"N", b"N", Dl * d, Er, Dr, a, Dr, t, Er, u, Er)
        # t'[l, f] = sum_(s, e) u[l, (s, e)] conj(b[f, (s, e)])
        tn = empty((Dl, El))
        _zgemm(b"N", b"H", Dl, El, d * Er, u, d * Er, b, d * Er, tn, El)
        t = tn
    assert tuple(t.shape) == (1, 1)
    return complex(t.reshape(-1)[0].item())


def mps_norm(psi):
    """(pytenet/mps.py:453-457)"""
    return float(np.sqrt(mps_vdot(psi, psi).real))


def apply_mpo(op, psi):
    """MPO applied to an MPS (pytenet/chain_ops.py:215-234), contracted on the GPU:
    per site out[(chi_l, D_l), s, (chi_r, D_r)] = sum_t W[chi_l, s, t, chi_r] A[D_l, t, D_r]
    as one complex GEMM over the physical index (operands laid out by device
    gathers), the grouping of the virtual bonds by a final gather. Bond quantum
    numbers are the pairwise flattening of (op, psi); returns a host MPS like the
    reference."""
    from .mps import MPS
    from .qnumber import qnumber_flatten, is_qsparse
    assert np.array_equal(np.asarray(psi.qsite), np.asarray(op.qsite))
    assert len(psi.a) == len(op.a)
    n = len(psi.a)
    qbonds = [qnumber_flatten((np.asarray(op.qbonds[i]), np.asarray(psi.qbonds[i])))
              for i in range(n + 1)]
    out = MPS(psi.qsite, qbonds, fill="postpone")
    L, st = lib(), stream_ptr()

    def gather(src, rows, cols, nr, nc):
        ro = torch.as_tensor(rows, dtype=torch.int64, device=device())
        co = torch.as_tensor(cols, dtype=torch.int64, device=device())
        dst = empty((nr, nc))
        call(L.ptn_gather, ptr(src), ptr(ro), ptr(co), nr, nc, ptr(dst), st)
        return dst

    tensors = []
    for i in range(n):
        w = to_dev(op.a[i])                                 # (cl, d, d, cr)
        a = to_dev(psi.a[i])                                # (Dl, d, Dr)
        cl, d, _, cr = op.a[i].shape
        Dl, _, Dr = psi.a[i].shape
        # Wm[(cl, s, cr), t] = W[cl, s, t, cr]
        ic, isd, ir = np.meshgrid(np.arange(cl), np.arange(d), np.arange(cr), indexing="ij")
        wrows = (ic * d * d * cr + isd * d * cr + ir).reshape(-1)
        wm = gather(w, wrows, np.arange(d) * cr, cl * d * cr, d)
        # At[t, (Dl, Dr)] = A[Dl, t, Dr]
        il, jr = np.meshgrid(np.arange(Dl), np.arange(Dr), indexing="ij")
        at = gather(a, np.arange(d) * Dr, (il * d * Dr + jr).reshape(-1), d, Dl * Dr)
        # X[(cl, s, cr), (Dl, Dr)] = Wm . At
        x = empty((cl * d * cr, Dl * Dr))
        _zgemm(b"N", b"N", cl * d * cr, Dl * Dr, d, wm, d, at, Dl * Dr, x, Dl * Dr)
        # out[(cl, Dl, s), (cr, Dr)] = X[cl, s, cr, Dl, Dr]
        jc, jl, js = np.meshgrid(np.arange(cl), np.arange(Dl), np.arange(d), indexing="ij")
        orows = (jc * d * cr * Dl * Dr + js * cr * Dl * Dr + jl * Dr).reshape(-1)
        kc, kr = np.meshgrid(np.arange(cr), np.arange(Dr), indexing="ij")
        ocols = (kc * Dl * Dr + kr).reshape(-1)
        t = gather(x, orows, ocols, cl * Dl * d, cr * Dr)
        tensors.append(t.view(cl * Dl, d, cr * Dr))
    out.a = [to_host(t).copy() for t in tensors]
    for i in range(n):
        assert is_qsparse(out.a[i], [out.qbonds[i], out.qsite, -out.qbonds[i + 1]]), \
            "sparsity pattern of MPS tensor does not match quantum numbers"
    return out
