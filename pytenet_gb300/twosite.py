"""
Two-site TDVP and DMRG on the GPU, drop-ins for pytenet.tdvp_twosite
(pytenet/tdvp.py:121-220) and pytenet.dmrg_twosite (pytenet/dmrg.py:96-178).

A local step works on the merged pair tensor (Dl, d*d, Dr) with the merged MPO pair
(chil, d*d, d*d, chir): the same fused Krylov entry points as the single-site sweep
(ptn_expm_site / ptn_eigh_site) with a physical dimension of d*d. The pair is split
by the block-sparse SVD on the device (ptn_svd per quantum-number block) and
truncated by the reference's rule; the new bond dimension and its quantum numbers
are decided on the host from the singular values, exactly as the reference does,
so bonds can grow and shrink. Site tensors and environments are device tensors
whose shapes follow the bonds; nothing is read back inside a sweep except the
singular values of each split.
"""

import warnings

import numpy as np
import torch

from . import _lib
from .block_sparse import Flip3, QRScratch, RowMajor, ColMajor, qr_execute, svd_execute, \
    take_singular, _svd_scratch
from .bond_ops import retained_bond_indices
from .device import Workspace, call, device, empty, lib, ptr, stream_ptr, to_dev, to_host
from .engine import MIXED_MIN_BOND, prec_code
from .qnumber import is_qsparse, qnumber_flatten, qr_plan

__all__ = ["tdvp_twosite", "dmrg_twosite", "merge_mpo_pair", "TwoSiteRun"]


def merge_mpo_pair(w0, w1):
    """Merged MPO tensor of two neighbouring sites, out[b0, (o0, o1), (i0, i1), b2] =
    sum_c w0[b0, o0, i0, c] w1[c, o1, i1, b2] (pytenet/mpo.py:314-322); host-side
    input preparation of a few hundred entries."""
    w0, w1 = np.asarray(w0), np.asarray(w1)
    a = np.tensordot(w0, w1, (3, 0))                 # (b0, o0, i0, o1, i1, b2)
    a = a.transpose((0, 1, 3, 2, 4, 5))
    s = a.shape
    return a.reshape((s[0], s[1] * s[2], s[3] * s[4], s[5]))


class TwoSiteRun:
    """Device state of a two-site TDVP / DMRG run."""

    def __init__(self, op, psi, numiter, precision="fp64"):
        n = len(op.a)
        assert n == len(psi.a) and n >= 2
        self.n = n
        self.numiter = int(numiter)
        if not 1 <= self.numiter < _lib.KRYLOV_MAXITER:
            raise ValueError(f"numiter_lanczos must be in [1, {_lib.KRYLOV_MAXITER})")
        self.prec = prec_code(precision)
        self.qsite = np.asarray(psi.qsite).copy()
        self.d = len(self.qsite)
        self.op_qbonds = [np.asarray(q) for q in op.qbonds]
        self.w = [to_dev(np.asarray(x, dtype=complex)) for x in op.a]
        self.h2 = [to_dev(merge_mpo_pair(op.a[i], op.a[i + 1])) for i in range(n - 1)]
        self.chi = [int(x.shape[0]) for x in op.a] + [int(op.a[-1].shape[3])]
        self.state = torch.zeros(lib().ptn_krylov_state_bytes(), dtype=torch.uint8,
                                 device=device())
        self.V = Workspace()
        self.ws = Workspace()
        self.gws = Workspace()
        self.qr_scratch = QRScratch()
        self.load(psi)

    # ------------------------------------------------------------ state
    def load(self, psi):
        self.a = [to_dev(x) for x in psi.a]
        self.qbonds = [np.asarray(q).copy() for q in psi.qbonds]

    def download(self, psi):
        psi.a = [to_host(x).copy() for x in self.a]
        psi.qbonds = [q.copy() for q in self.qbonds]

    def prec_for(self, Dl, Dr):
        if self.prec != _lib.PREC_FP64 and min(Dl, Dr) < MIXED_MIN_BOND:
            return _lib.PREC_FP64
        return self.prec

    # ------------------------------------------------------------ environments
    def init_envs(self):
        """lblocks[0] = [[[1]]] and all right blocks (pytenet/chain_ops.py:102-113)."""
        n = self.n
        self.lenv = [None] * n
        self.renv = [None] * n
        self.lenv[0] = torch.ones((1, 1, 1), dtype=torch.complex128, device=device())
        self.renv[n - 1] = torch.ones((1, 1, 1), dtype=torch.complex128, device=device())
        for i in reversed(range(n - 1)):
            self.env_right(i + 1)

    def check_envs(self):
        """is_qsparse check of the right blocks (pytenet/tdvp.py:60-63)."""
        for i in range(self.n):
            assert is_qsparse(to_host(self.renv[i]), [self.qbonds[i + 1], self.op_qbonds[i + 1],
                                                      -self.qbonds[i + 1]]), \
                "sparsity pattern of operator blocks must match quantum numbers"

    def env_left(self, i):
        """lblocks[i+1] = contraction_operator_step_left(a, a, w, lblocks[i])."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.a[i].shape
        cl, cr = self.chi[i], self.chi[i + 1]
        out = empty((Dr, cr, Dr))
        prec = self.prec_for(Dl, Dr)
        wsb = L.ptn_env_workspace_bytes(Dl, d, Dr, cl, cr, prec)
        ws = self.ws.get(wsb)
        call(L.ptn_env_step_left, ptr(self.a[i]), ptr(self.a[i]), ptr(self.w[i]),
             ptr(self.lenv[i]), ptr(out), Dl, d, Dr, cl, cr, prec, ptr(ws), wsb, st)
        self.lenv[i + 1] = out

    def env_right(self, i):
        """rblocks[i-1] = contraction_operator_step_right(a, a, w, rblocks[i])."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.a[i].shape
        cl, cr = self.chi[i], self.chi[i + 1]
        out = empty((Dl, cl, Dl))
        prec = self.prec_for(Dl, Dr)
        wsb = L.ptn_env_workspace_bytes(Dl, d, Dr, cl, cr, prec)
        ws = self.ws.get(wsb)
        call(L.ptn_env_step_right, ptr(self.a[i]), ptr(self.a[i]), ptr(self.w[i]),
             ptr(self.renv[i]), ptr(out), Dl, d, Dr, cl, cr, prec, ptr(ws), wsb, st)
        self.renv[i - 1] = out

    # ------------------------------------------------------------ local steps
    def _krylov_buffers(self, nvec):
        return self.V.get((self.numiter + 1) * nvec * 16)

    def local_expm(self, x, w, l, r, cl, cr, dt):
        """x <- expm(-dt H_eff) x in place (_local_hamiltonian_step, tdvp.py:223-229)
        for a site tensor x (Dl, dd, Dr) and MPO tensor w (cl, dd, dd, cr)."""
        L, st = lib(), stream_ptr()
        Dl, dd, Dr = x.shape
        z = -complex(dt)
        prec = self.prec_for(Dl, Dr)
        wsb = L.ptn_site_step_workspace_bytes(Dl, dd, Dr, cl, cr, prec)
        ws = self.ws.get(wsb)
        V = self._krylov_buffers(Dl * dd * Dr)
        call(L.ptn_expm_site, ptr(x), ptr(w), ptr(l), ptr(r), Dl, dd, Dr, cl, cr, z.real, z.imag,
             self.numiter, prec, ptr(V), ptr(self.state), ptr(ws), wsb, st)

    def local_eigh(self, x, w, l, r, cl, cr):
        """x <- lowest Ritz vector of H_eff (_minimize_local_energy, dmrg.py:181-189)."""
        L, st = lib(), stream_ptr()
        Dl, dd, Dr = x.shape
        prec = self.prec_for(Dl, Dr)
        wsb = L.ptn_site_step_workspace_bytes(Dl, dd, Dr, cl, cr, prec)
        ws = self.ws.get(wsb)
        V = self._krylov_buffers(Dl * dd * Dr)
        call(L.ptn_eigh_site, ptr(x), ptr(w), ptr(l), ptr(r), Dl, dd, Dr, cl, cr, self.numiter,
             prec, ptr(V), ptr(self.state), ptr(ws), wsb, st)

    def merged(self, i):
        """mps_merge_tensor_pair(a[i], a[i+1]) (pytenet/mps.py:528-535): one GEMM."""
        L, st = lib(), stream_ptr()
        Dl, d0, Dm = self.a[i].shape
        Dm2, d1, Dr = self.a[i + 1].shape
        assert Dm == Dm2
        out = empty((Dl, d0 * d1, Dr))
        M, N, K = Dl * d0, d1 * Dr, Dm
        wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
        ws = self.gws.get(wsb)
        call(L.ptn_zgemm, b"N", b"N", M, N, K, _lib.cval(1), ptr(self.a[i]), K, 0,
             ptr(self.a[i + 1]), N, 0, _lib.cval(0), ptr(out), N, 0, 1, ptr(ws), wsb, st)
        return out

    def split(self, i, x, svd_distr, tol):
        """mps_split_tensor_svd (pytenet/mps.py:538-568) of the pair tensor x into
        a[i], a[i+1] with the new bond's quantum numbers; singular values go to
        the left or the right factor."""
        L, st = lib(), stream_ptr()
        Dl, dd, Dr = x.shape
        d = self.d
        q0 = qnumber_flatten([self.qbonds[i], self.qsite])
        q1 = qnumber_flatten([-self.qsite, self.qbonds[i + 2]])
        plan = qr_plan(q0, q1)
        u, s, vh = svd_execute(plan, x, RowMajor(d * Dr), _svd_scratch())
        s_host = s.cpu().numpy()          # the truncation is an integer decision
        idx = retained_bond_indices(s_host, tol)
        u, vh = take_singular(u, vh, idx)
        k = len(idx)
        sk = torch.from_numpy(np.ascontiguousarray(s_host[idx])).to(device())
        if k > 0:
            if svd_distr == "left":
                call(L.ptn_diag_scale, ptr(u), Dl * d, k, k, ptr(sk), 0, st)
            elif svd_distr == "right":
                call(L.ptn_diag_scale, ptr(vh), k, d * Dr, d * Dr, ptr(sk), 1, st)
            else:
                raise ValueError('`svd_distr` parameter must be "left" or "right".')
        self.a[i] = u.view(Dl, d, k)
        self.a[i + 1] = vh.view(k, d, Dr)
        self.qbonds[i + 1] = plan.qinterm[idx].copy()

    def right_qr_first(self):
        """psi.a[0] <- right-orthonormal Q of site 0, qbonds[0] updated; the R factor
        is discarded (the final step of pytenet/dmrg.py:96-178, via
        local_orthonormalize_right_qr, pytenet/mps.py:476-491)."""
        Dl, d, Dr = self.a[0].shape
        plan = qr_plan(qnumber_flatten((-self.qbonds[1], self.qsite)), -self.qbonds[0])
        K = plan.K
        src = self.a[0].reshape(-1).clone()
        q = empty((K * d * Dr,))
        c = empty((Dl * K,))
        qr_execute(plan, src, Flip3(d, Dr), q, Flip3(d, Dr), c, ColMajor(K), self.qr_scratch)
        self.a[0] = q.view(K, d, Dr)
        self.qbonds[0] = -plan.qinterm

    def eval0(self):
        off = _lib.KrylovState.eval0.offset
        return self.state[off:off + 8].view(torch.float64)

    def breakdowns(self):
        raw = bytes(self.state[: _lib.C.sizeof(_lib.KrylovState)].cpu().numpy())
        return _lib.KrylovState.from_buffer_copy(raw).breakdowns

    # ------------------------------------------------------------ sweeps
    def tdvp_step(self, dt, tol):
        """One symmetric two-site TDVP time step (pytenet/tdvp.py:150-218)."""
        n = self.n
        for i in range(n - 2):
            x = self.merged(i)
            self.local_expm(x, self.h2[i], self.lenv[i], self.renv[i + 1], self.chi[i],
                            self.chi[i + 2], 0.5 * dt)
            self.split(i, x, "right", tol)
            self.env_left(i)
            self.local_expm(self.a[i + 1], self.w[i + 1], self.lenv[i + 1], self.renv[i + 1],
                            self.chi[i + 1], self.chi[i + 2], -0.5 * dt)
        i = n - 2
        x = self.merged(i)
        self.local_expm(x, self.h2[i], self.lenv[i], self.renv[i + 1], self.chi[i],
                        self.chi[i + 2], dt)
        self.split(i, x, "left", tol)
        self.env_right(i + 1)
        for i in reversed(range(n - 2)):
            self.local_expm(self.a[i + 1], self.w[i + 1], self.lenv[i + 1], self.renv[i + 1],
                            self.chi[i + 1], self.chi[i + 2], -0.5 * dt)
            x = self.merged(i)
            self.local_expm(x, self.h2[i], self.lenv[i], self.renv[i + 1], self.chi[i],
                            self.chi[i + 2], 0.5 * dt)
            self.split(i, x, "left", tol)
            self.env_right(i + 1)

    def dmrg_sweep(self, en_out, k, tol):
        """One left and right two-site DMRG sweep (pytenet/dmrg.py:134-176); the
        Ritz value of its last local step goes to en_out[k] on the device."""
        n = self.n
        for i in range(n - 2):
            x = self.merged(i)
            self.local_eigh(x, self.h2[i], self.lenv[i], self.renv[i + 1], self.chi[i],
                            self.chi[i + 2])
            self.split(i, x, "right", tol)
            self.env_left(i)
        for i in reversed(range(n - 1)):
            x = self.merged(i)
            self.local_eigh(x, self.h2[i], self.lenv[i], self.renv[i + 1], self.chi[i],
                            self.chi[i + 2])
            self.split(i, x, "left", tol)
            self.env_right(i + 1)
        self.right_qr_first()
        en_out[k:k + 1].copy_(self.eval0())


def _warn(run):
    nb = run.breakdowns()
    if nb:
        warnings.warn(f"Lanczos iteration stopped early (beta ~= 0) in {nb} local step(s).",
                      RuntimeWarning, stacklevel=3)


def tdvp_twosite(hamiltonian, psi, dt, numsteps, numiter_lanczos=25, tol_split=0,
                 precision="fp64"):
    """Symmetric two-site TDVP; `psi` is overwritten in place (bond dimensions may
    change) and the norm of the initial `psi` is returned (pytenet/tdvp.py:121-220).
    All numerics run on the GPU."""
    nrm = psi.orthonormalize(mode="right")
    run = TwoSiteRun(hamiltonian, psi, numiter_lanczos, precision)
    run.init_envs()
    run.check_envs()
    for _ in range(numsteps):
        run.tdvp_step(dt, tol_split)
    run.download(psi)
    _warn(run)
    return nrm


def dmrg_twosite(hamiltonian, psi, numsweeps, numiter_lanczos=25, tol_split=0,
                 precision="fp64"):
    """Two-site DMRG; `psi` is overwritten in place; returns the energy after each
    sweep (pytenet/dmrg.py:96-178). All numerics run on the GPU."""
    psi.orthonormalize(mode="right")
    run = TwoSiteRun(hamiltonian, psi, numiter_lanczos, precision)
    run.init_envs()
    run.check_envs()
    en = torch.zeros(numsweeps, dtype=torch.float64, device=device())
    for k in range(numsweeps):
        run.dmrg_sweep(en, k, tol_split)
    run.download(psi)
    _warn(run)
    return en.cpu().numpy()
