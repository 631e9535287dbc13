"""
Krylov subspace methods with the signatures of pytenet/krylov.py (lanczos_iteration,
expm_krylov, eigh_krylov, eigh_tridiag) for a user-supplied operator `afunc`.

The vector recurrences, the breakdown rule (beta < 100 n eps) and the tridiagonal
eigenproblem run on the GPU (the ptn_krylov_* entry points). `afunc` is called
with the same kind of vector the caller passed in: NumPy arrays stay NumPy (a
host round trip per application, for drop-in use with host operators), CUDA
tensors stay on the device. The sweeps do not use this module; they call the
fused device steps that apply H_eff without leaving the GPU.
"""

import warnings

import numpy as np
import torch

from . import _lib
from .device import call, device, empty, lib, ptr, stream_ptr, to_dev, to_host

__all__ = ["lanczos_iteration", "expm_krylov", "eigh_krylov", "eigh_tridiag"]


class _Run:
    def __init__(self, vstart, numiter):
        if not 1 <= numiter < _lib.KRYLOV_MAXITER:
            raise ValueError(f"numiter must be in [1, {_lib.KRYLOV_MAXITER})")
        self.host = not isinstance(vstart, torch.Tensor)
        v = to_dev(vstart).reshape(-1)
        self.n = v.numel()
        self.numiter = numiter
        self.V = empty(((numiter + 1), self.n))
        self.state = torch.zeros(lib().ptn_krylov_state_bytes(), dtype=torch.uint8, device=device())
        call(lib().ptn_krylov_start, ptr(self.state), ptr(v), ptr(self.V), self.n, numiter,
             stream_ptr())
        self.vstart = v

    def read_state(self):
        raw = self.state[: _lib.C.sizeof(_lib.KrylovState)].cpu().numpy().tobytes()
        return _lib.KrylovState.from_buffer_copy(raw)

    def apply(self, afunc, j, out_row):
        x = self.V[j]
        y = afunc(to_host(x) if self.host else x)
        self.V[out_row].copy_(to_dev(np.asarray(y) if self.host else y).reshape(-1))

    def run(self, afunc):
        L, st = lib(), stream_ptr()
        s = self.read_state()
        assert s.status == _lib.PTN_OK and s.nrm > 0
        m = self.numiter
        for j in range(m - 1):
            self.apply(afunc, j, j + 1)
            call(L.ptn_krylov_step, ptr(self.state), ptr(self.V), self.n, j, st)
            s = self.read_state()
            if s.stopped:
                warnings.warn(f"beta[{j}] ~= 0 encountered during Lanczos iteration.",
                              RuntimeWarning, stacklevel=3)
                return s
        self.apply(afunc, m - 1, m)
        call(L.ptn_krylov_last, ptr(self.state), ptr(self.V), ptr(self.V[m]), self.n, m - 1, st)
        return self.read_state()


def lanczos_iteration(afunc, vstart, numiter):
    """Matrix-free Lanczos (pytenet/krylov.py:12-57); returns (alpha, beta, V)
    with V of shape (len(vstart), m_used)."""
    r = _Run(vstart, numiter)
    s = r.run(afunc)
    m = s.m_used
    alpha = np.array(s.alpha[:m])
    beta = np.array(s.beta[:m - 1])
    v = r.V[:m].T
    return alpha, beta, (to_host(v) if r.host else v)


def _tridiag_eig(r, m):
    ev = torch.empty(m, dtype=torch.float64, device=device())
    U = torch.empty((m, m), dtype=torch.float64, device=device())
    call(lib().ptn_krylov_tridiag_eig, ptr(r.state), ptr(ev), ptr(U), stream_ptr())
    return ev, U


def eigh_tridiag(d, e):
    """Eigen-decomposition of the real symmetric tridiagonal matrix with diagonal
    d and off-diagonal e (pytenet/krylov.py:142-150), computed on the GPU."""
    d = np.asarray(d, dtype=float)
    e = np.asarray(e, dtype=float)
    m = len(d)
    if not 1 <= m < _lib.KRYLOV_MAXITER:
        raise ValueError("tridiagonal size out of range")
    st = _lib.KrylovState()
    st.m_used = m
    st.maxiter = m
    st.nrm = 1.0
    for i in range(m):
        st.alpha[i] = d[i]
    for i in range(m - 1):
        st.beta[i] = e[i]
    raw = bytearray(lib().ptn_krylov_state_bytes())
    raw[: _lib.C.sizeof(st)] = bytes(st)
    state = torch.frombuffer(raw, dtype=torch.uint8).to(device())

    class _R:
        pass
    rr = _R()
    rr.state = state
    ev, U = _tridiag_eig(rr, m)
    return to_host(ev), to_host(U)


def eigh_krylov(afunc, vstart, numiter, numeig):
    """Lowest Ritz pairs (pytenet/krylov.py:110-119)."""
    r = _Run(vstart, numiter)
    s = r.run(afunc)
    m = s.m_used
    ev, U = _tridiag_eig(r, m)
    Uc = U[:, :numeig].to(torch.complex128).contiguous()
    # u_ritz = V^T U[:, :numeig]  (n x numeig)
    out = empty((r.n, numeig))
    L = lib()
    wsb = L.ptn_zgemm_workspace_bytes(r.n, numeig, m, 1)
    ws = torch.empty(max(wsb, 256), dtype=torch.uint8, device=device())
    call(L.ptn_zgemm, b"T", b"N", r.n, numeig, m, _lib.cval(1), ptr(r.V), r.n, 0, ptr(Uc), numeig,
         0, _lib.cval(0), ptr(out), numeig, 0, 1, ptr(ws), wsb, stream_ptr())
    w = to_host(ev[:numeig])
    return w, (to_host(out) if r.host else out)


def expm_krylov(afunc, vec, dt, numiter, hermitian=False):
    """Krylov approximation of expm(dt A) vec (pytenet/krylov.py:122-139). Only
    the Hermitian (Lanczos) branch is provided: the single-site sweeps always
    take it (pytenet/tdvp.py:229,237)."""
    if not hermitian:
        raise NotImplementedError("expm_krylov: only hermitian=True (Lanczos) is provided")
    r = _Run(vec, numiter)
    r.run(afunc)
    z = complex(dt)
    L, st = lib(), stream_ptr()
    call(L.ptn_krylov_expm_coef, ptr(r.state), z.real, z.imag, st)
    out = empty((r.n,))
    call(L.ptn_krylov_combine, ptr(r.state), ptr(r.V), r.n, ptr(out), st)
    return to_host(out) if r.host else out
