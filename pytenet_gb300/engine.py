"""
Device sweep engine for single-site TDVP and DMRG (pytenet/tdvp.py:26-118,
pytenet/dmrg.py:22-93).

State lives in HBM for the whole run: one storage buffer per site tensor (sized
at the initial bond dimensions; single-site sweeps never grow a bond), the MPO
tensors (complex128), the left / right environments, the Lanczos basis, the
Krylov state and the scratch of the contractions and of the QR. The host keeps
only integers: the logical shape of every site tensor and the quantum numbers,
which it updates from the QR plans exactly like the reference does. Every
numerical step is one or a few C-ABI calls that enqueue kernels on the current
stream; nothing synchronises inside a sweep, so a whole time step can be
captured in a CUDA graph and replayed.
"""

import warnings

import numpy as np
import torch

from . import _lib
from .block_sparse import ColMajor, Flip3, QRScratch, RowMajor, qr_execute
from .device import CDT, Workspace, call, device, empty, lib, ptr, stream_ptr, to_dev, to_host
from .qnumber import is_qsparse, qnumber_flatten, qr_plan

PREC = {"fp64": _lib.PREC_FP64, "plain": _lib.PREC_FP64, "mixed": _lib.PREC_SPLIT_BF16,
        "split-bf16": _lib.PREC_SPLIT_BF16}
# smallest bond dimension (both sides) at which the mixed form uses the tensor cores
MIXED_MIN_BOND = 32


def prec_code(precision):
    if isinstance(precision, int):
        return precision
    try:
        return PREC[precision]
    except KeyError:
        raise ValueError(f"precision must be one of {sorted(PREC)}") from None


class DeviceMPS:
    """Device-resident MPS: site tensors plus host-side integer quantum numbers."""

    def __init__(self, psi):
        self.nsites = len(psi.a)
        self.qsite = np.asarray(psi.qsite).copy()
        self.qbonds = [np.asarray(q).copy() for q in psi.qbonds]
        self.d = len(self.qsite)
        self.shape = [tuple(int(s) for s in x.shape) for x in psi.a]
        self.buf = []
        for x in psi.a:
            t = to_dev(x).reshape(-1)
            self.buf.append(t)
        self.maxsize = max(t.numel() for t in self.buf)
        self.tmp = empty((self.maxsize,))
        self.work = empty((self.maxsize,))
        self.cbuf = empty((self.maxsize,))
        self.rbuf = empty((self.maxsize,))
        self.qr_ws = Workspace()
        self.gemm_ws = Workspace()
        self.scratch = QRScratch()
        self.nrm_dev = torch.zeros(1, dtype=torch.float64, device=device())
        self.one = torch.ones(1, dtype=CDT, device=device())

    # ---------------------------------------------------------------- views
    def site(self, i):
        s = self.shape[i]
        return self.buf[i][: s[0] * s[1] * s[2]].view(s)

    def download(self, psi):
        for i in range(self.nsites):
            psi.a[i] = to_host(self.site(i)).copy()
        psi.qbonds = [q.copy() for q in self.qbonds]

    # ---------------------------------------------------------------- QR steps
    def qr_left(self, i):
        """Left-orthonormalise site i (pytenet/tdvp.py:72-77, mps.py:460-473).
        Returns the R factor C (K x Dr) as a device view; updates shape / qbonds."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        m, n = Dl * d, Dr
        plan = qr_plan(qnumber_flatten((self.qbonds[i], self.qsite)), self.qbonds[i + 1])
        K = plan.K
        c = self.cbuf[: K * n].view(K, n)
        a = self.buf[i]
        if plan.dense:
            wsb = L.ptn_qr_workspace_bytes(m, n)
            ws = self.qr_ws.get(wsb)
            call(L.ptn_qr, ptr(a), m, n, ptr(a), K, ptr(c), n, ptr(ws), wsb, st)
        else:
            src = self.tmp[: m * n]
            src.copy_(a[: m * n])
            qr_execute(plan, src, RowMajor(n), a[: m * K], RowMajor(K), c, RowMajor(n),
                       self.scratch)
        self.shape[i] = (Dl, d, K)
        self.qbonds[i + 1] = plan.qinterm.copy()
        return c

    def qr_right(self, i):
        """Right-orthonormalise site i via the QR of its (2,1,0) transpose
        (pytenet/tdvp.py:95-104, mps.py:476-491). Returns C = R^T (Dl x K)."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        m, n = Dr * d, Dl
        plan = qr_plan(qnumber_flatten((-self.qbonds[i + 1], self.qsite)), -self.qbonds[i])
        K = plan.K
        c = self.cbuf[: n * K].view(n, K)
        a = self.buf[i]
        if plan.dense:
            work = self.work[: m * n]
            call(L.ptn_transpose_210, ptr(a), ptr(work), Dl, d, Dr, st)
            wsb = L.ptn_qr_workspace_bytes(m, n)
            ws = self.qr_ws.get(wsb)
            r = self.rbuf[: K * n]
            call(L.ptn_qr, ptr(work), m, n, ptr(work), K, ptr(r), n, ptr(ws), wsb, st)
            call(L.ptn_transpose_210, ptr(work), ptr(a), Dr, d, K, st)
            call(L.ptn_transpose_210, ptr(r), ptr(c), K, 1, n, st)
        else:
            src = self.tmp[: Dl * d * Dr]
            src.copy_(a[: Dl * d * Dr])
            qr_execute(plan, src, Flip3(d, Dr), a[: K * d * Dr], Flip3(d, Dr), c, ColMajor(K),
                       self.scratch)
        self.shape[i] = (K, d, Dr)
        self.qbonds[i] = -plan.qinterm
        return c

    def _gemm(self, M, N, K, a, b, out, mixed):
        """out (M x N) = a (M x K) b (K x N), row-major complex: FP64 DMMA, or with
        mixed=True the tensor-core digit GEMM (the contraction arithmetic of the
        mixed form)."""
        L, st = lib(), stream_ptr()
        if mixed:
            wsb = L.ptn_zgemm_split_bf16_workspace_bytes(M, N, K)
            ws = self.gemm_ws.get(wsb)
            call(L.ptn_zgemm_split_bf16, ptr(a), K, ptr(b), N, ptr(out), N, M, N, K, ptr(ws),
                 wsb, st)
            return
        wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
        ws = self.gemm_ws.get(wsb)
        call(L.ptn_zgemm, b"N", b"N", M, N, K, _lib.cval(1), ptr(a), K, 0, ptr(b), N, 0,
             _lib.cval(0), ptr(out), N, 0, 1, ptr(ws), wsb, st)

    def absorb_left(self, c, i, mixed=False):
        """psi.a[i] = tensordot(c, psi.a[i], (1, 0)) (pytenet/tdvp.py:84)."""
        K, n = c.shape
        Dl, d, Dr = self.shape[i]
        assert n == Dl
        out = self.tmp[: K * d * Dr]
        self._gemm(K, d * Dr, n, c, self.buf[i], out, mixed)
        self.buf[i][: K * d * Dr].copy_(out)
        self.shape[i] = (K, d, Dr)

    def absorb_right(self, c, i, mixed=False):
        """psi.a[i] = tensordot(psi.a[i], c, (2, 0)) (pytenet/tdvp.py:112)."""
        n, K = c.shape
        Dl, d, Dr = self.shape[i]
        assert n == Dr
        out = self.tmp[: Dl * d * K]
        self._gemm(Dl * d, K, n, self.buf[i], c, out, mixed)
        self.buf[i][: Dl * d * K].copy_(out)
        self.shape[i] = (Dl, d, K)

    def orthonormalize(self, mode="left"):
        """MPS.orthonormalize on the device (pytenet/mps.py:141-178). Returns the
        norm as a device scalar (float64 tensor); no host synchronisation."""
        L, st = lib(), stream_ptr()
        if self.nsites == 0:
            self.nrm_dev.fill_(1.0)
            return self.nrm_dev
        if mode == "left":
            for i in range(self.nsites - 1):
                c = self.qr_left(i)
                self.absorb_left(c, i + 1)
            i = self.nsites - 1
            c = self.qr_left(i)   # R (1 x 1): the norm
            call(L.ptn_sign_fix, ptr(self.buf[i]), int(np.prod(self.shape[i])), ptr(c),
                 ptr(self.nrm_dev), st)
            return self.nrm_dev
        if mode == "right":
            for i in reversed(range(1, self.nsites)):
                c = self.qr_right(i)
                self.absorb_right(c, i - 1)
            c = self.qr_right(0)
            call(L.ptn_sign_fix, ptr(self.buf[0]), int(np.prod(self.shape[0])), ptr(c),
                 ptr(self.nrm_dev), st)
            return self.nrm_dev
        raise ValueError(f'`mode` = {mode} invalid; must be "left" or "right".')


class DepthState:
    """Device buffers of the learned Lanczos depth: per-(site, kind) history of
    the previous alpha / beta, the MLP parameters (or None: fixed depth, or with
    check_from > 0 the residual-only criterion tested from that depth on), and an
    optional training-record log."""

    def __init__(self, nsites, params=None, tol=1e-10, log_capacity=0, check_from=0):
        self.history = torch.zeros((2 * nsites, 8), dtype=torch.float32, device=device())
        self.params = params
        self.tol = float(tol)
        self.log = None
        self.log_count = None
        self.log_capacity = int(log_capacity)
        if log_capacity > 0:
            self.log = torch.zeros((log_capacity, _lib.DEPTH_RECORD), dtype=torch.float64,
                                   device=device())
            self.log_count = torch.zeros(1, dtype=torch.int32, device=device())
        self.nsites = nsites
        self.check_from = int(check_from)

    def ctx(self, site, kind):
        c = _lib.DepthCtx()
        c.params = ptr(self.params) if self.params is not None else None
        c.history = ptr(self.history)
        c.slot = 2 * site + kind
        c.site = site
        c.nsites = self.nsites
        c.kind = kind
        c.tol = self.tol
        c.log = ptr(self.log) if self.log is not None else None
        c.log_count = ptr(self.log_count) if self.log_count is not None else None
        c.log_capacity = self.log_capacity
        c.check_from = self.check_from
        return c

    def records(self):
        n = min(int(self.log_count.item()), self.log_capacity)
        return self.log[:n]


class Chain(DeviceMPS):
    """Device state of one TDVP / DMRG run: MPS, MPO, environments, Krylov buffers."""

    def __init__(self, op, psi, numiter, precision="fp64", depth=None, mixed_min_bond=None):
        assert len(op.a) == len(psi.a)
        super().__init__(psi)
        self.prec = prec_code(precision)
        self.mixed_min_bond = MIXED_MIN_BOND if mixed_min_bond is None else int(mixed_min_bond)
        self.numiter = int(numiter)
        if not 1 <= self.numiter < _lib.KRYLOV_MAXITER:
            raise ValueError(f"numiter_lanczos must be in [1, {_lib.KRYLOV_MAXITER})")
        self.op_qbonds = [np.asarray(q) for q in op.qbonds]
        self.w = [to_dev(x) for x in op.a]
        self.chi = [int(x.shape[0]) for x in op.a] + [int(op.a[-1].shape[3])]
        Lx = self.nsites
        bd = [s[0] for s in self.shape] + [self.shape[-1][2]]
        # environments: lenv[i] (b_i, chi_i, b_i), renv[i] (b_{i+1}, chi_{i+1}, b_{i+1})
        self.lenv = [empty((bd[i] * self.chi[i] * bd[i],)) for i in range(Lx)]
        self.renv = [empty((bd[i + 1] * self.chi[i + 1] * bd[i + 1],)) for i in range(Lx)]
        self.lshape = [None] * Lx
        self.rshape = [None] * Lx
        nmax = max(int(np.prod(s)) for s in self.shape)
        self.V = empty(((self.numiter + 1) * nmax,))
        self.state = torch.zeros(lib().ptn_krylov_state_bytes(), dtype=torch.uint8, device=device())
        self.cws = Workspace()
        L = lib()
        need = 0
        for i in range(Lx):
            Dl, d, Dr = self.shape[i]
            cl, cr = self.chi[i], self.chi[i + 1]
            for p in {self.prec, _lib.PREC_FP64}:
                need = max(need, L.ptn_site_step_workspace_bytes(Dl, d, Dr, cl, cr, p),
                           L.ptn_env_workspace_bytes(Dl, d, Dr, cl, cr, p),
                           L.ptn_bond_step_workspace_bytes(Dr, Dr, cr, p),
                           L.ptn_bond_step_workspace_bytes(Dl, Dl, cl, p))
        self.cws_bytes = need
        self.cws.get(need)
        self.depth = depth

    def prec_for(self, Dl, Dr):
        """Arithmetic of one local problem. The mixed form runs the tensor-core digit
        GEMMs only where both bonds reach mixed_min_bond (MIXED_MIN_BOND unless set):
        below that the contractions are too small to fill a 128 x 96 tile, and the
        Krylov space of a small problem can be exhausted (a Lanczos breakdown at
        beta < 100 n eps), which only the FP64 operator detects the way the reference
        does. The batched driver raises it per bucket: a tensor-core GEMM CTA takes a
        whole SM's shared memory and tensor memory, so small problems of concurrent
        instances overlap better on the FP64 path."""
        if self.prec != _lib.PREC_FP64 and min(Dl, Dr) < self.mixed_min_bond:
            return _lib.PREC_FP64
        return self.prec

    # ---------------------------------------------------------------- envs
    def lview(self, i):
        s = self.lshape[i]
        return self.lenv[i][: s[0] * s[1] * s[2]].view(s)

    def rview(self, i):
        s = self.rshape[i]
        return self.renv[i][: s[0] * s[1] * s[2]].view(s)

    def init_envs(self):
        """lblocks[0] = [[[1]]] and all right blocks (pytenet/chain_ops.py:102-113)."""
        Lx = self.nsites
        self.lshape[0] = (1, 1, 1)
        self.lenv[0][:1].fill_(1.0)
        self.rshape[Lx - 1] = (1, 1, 1)
        self.renv[Lx - 1][:1].fill_(1.0)
        for i in reversed(range(Lx - 1)):
            self.env_right(i + 1)

    def check_envs(self):
        """is_qsparse consistency check of the right blocks (pytenet/tdvp.py:60-63)."""
        for i in range(self.nsites):
            assert is_qsparse(self.rview(i), [self.qbonds[i + 1], self.op_qbonds[i + 1],
                                              -self.qbonds[i + 1]]), \
                "sparsity pattern of operator blocks must match quantum numbers"

    def env_left(self, i):
        """lblocks[i+1] = contraction_operator_step_left(a, a, w, lblocks[i])."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        cl, cr = self.chi[i], self.chi[i + 1]
        assert self.lshape[i] == (Dl, cl, Dl)
        a = self.buf[i]
        ws = self.cws.get(self.cws_bytes)
        call(L.ptn_env_step_left, ptr(a), ptr(a), ptr(self.w[i]), ptr(self.lenv[i]),
             ptr(self.lenv[i + 1]), Dl, d, Dr, cl, cr, self.prec_for(Dl, Dr), ptr(ws),
             self.cws_bytes, st)
        self.lshape[i + 1] = (Dr, cr, Dr)

    def env_right(self, i):
        """rblocks[i-1] = contraction_operator_step_right(a, a, w, rblocks[i])."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        cl, cr = self.chi[i], self.chi[i + 1]
        assert self.rshape[i] == (Dr, cr, Dr)
        a = self.buf[i]
        ws = self.cws.get(self.cws_bytes)
        call(L.ptn_env_step_right, ptr(a), ptr(a), ptr(self.w[i]), ptr(self.renv[i]),
             ptr(self.renv[i - 1]), Dl, d, Dr, cl, cr, self.prec_for(Dl, Dr), ptr(ws),
             self.cws_bytes, st)
        self.rshape[i - 1] = (Dl, cl, Dl)

    # ---------------------------------------------------------------- local steps
    def site_expm(self, i, dt):
        """psi.a[i] = expm(-dt H_eff) psi.a[i] (_local_hamiltonian_step, tdvp.py:223-229)."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        cl, cr = self.chi[i], self.chi[i + 1]
        z = -complex(dt)
        prec = self.prec_for(Dl, Dr)
        ws = self.cws.get(self.cws_bytes)
        if self.depth is not None:
            ctx = self.depth.ctx(i, 0)
            call(L.ptn_expm_site_ex, ptr(self.buf[i]), ptr(self.w[i]), ptr(self.lenv[i]),
                 ptr(self.renv[i]), Dl, d, Dr, cl, cr, z.real, z.imag, self.numiter, prec,
                 _lib.C.byref(ctx), ptr(self.V), ptr(self.state), ptr(ws), self.cws_bytes, st)
            return
        call(L.ptn_expm_site, ptr(self.buf[i]), ptr(self.w[i]), ptr(self.lenv[i]),
             ptr(self.renv[i]), Dl, d, Dr, cl, cr, z.real, z.imag, self.numiter, prec,
             ptr(self.V), ptr(self.state), ptr(ws), self.cws_bytes, st)

    def bond_expm(self, c, l, r, chi, dt, site=0):
        """c = expm(-dt H_bond) c (_local_bond_step, tdvp.py:232-238)."""
        L, st = lib(), stream_ptr()
        Dl, Dr = c.shape
        z = -complex(dt)
        prec = self.prec_for(Dl, Dr)
        ws = self.cws.get(self.cws_bytes)
        if self.depth is not None:
            ctx = self.depth.ctx(site, 1)
            call(L.ptn_expm_bond_ex, ptr(c), ptr(l), ptr(r), Dl, Dr, chi, z.real, z.imag,
                 self.numiter, prec, _lib.C.byref(ctx), ptr(self.V), ptr(self.state),
                 ptr(ws), self.cws_bytes, st)
            return
        call(L.ptn_expm_bond, ptr(c), ptr(l), ptr(r), Dl, Dr, chi, z.real, z.imag, self.numiter,
             prec, ptr(self.V), ptr(self.state), ptr(ws), self.cws_bytes, st)

    def site_eigh(self, i):
        """Lowest Ritz vector of H_eff (_minimize_local_energy, dmrg.py:181-189)."""
        L, st = lib(), stream_ptr()
        Dl, d, Dr = self.shape[i]
        cl, cr = self.chi[i], self.chi[i + 1]
        ws = self.cws.get(self.cws_bytes)
        call(L.ptn_eigh_site, ptr(self.buf[i]), ptr(self.w[i]), ptr(self.lenv[i]),
             ptr(self.renv[i]), Dl, d, Dr, cl, cr, self.numiter, self.prec_for(Dl, Dr),
             ptr(self.V),
             ptr(self.state), ptr(ws), self.cws_bytes, st)

    # ---------------------------------------------------------------- sweeps
    def mixed_absorb(self, c, i):
        """Whether absorbing the bond matrix c into site i runs on the tensor cores:
        the mixed form, with every dimension of the product at least mixed_min_bond."""
        if self.prec == _lib.PREC_FP64:
            return False
        Dl, d, Dr = self.shape[i]
        return min(c.shape[0], c.shape[1], Dl, Dr) >= self.mixed_min_bond

    def tdvp_step(self, dt):
        """One symmetric single-site TDVP time step (pytenet/tdvp.py:65-115)."""
        n = self.nsites
        for i in range(n - 1):
            self.site_expm(i, 0.5 * dt)
            c = self.qr_left(i)
            self.env_left(i)
            self.bond_expm(c, self.lenv[i + 1], self.renv[i], self.chi[i + 1], -0.5 * dt, site=i)
            self.absorb_left(c, i + 1, self.mixed_absorb(c, i + 1))
        self.site_expm(n - 1, dt)
        for i in reversed(range(1, n)):
            c = self.qr_right(i)
            self.env_right(i)
            self.bond_expm(c, self.lenv[i], self.renv[i - 1], self.chi[i], -0.5 * dt, site=i - 1)
            self.absorb_right(c, i - 1, self.mixed_absorb(c, i - 1))
            self.site_expm(i - 1, 0.5 * dt)

    def dmrg_sweep(self, en_out, k):
        """One left and right DMRG sweep (pytenet/dmrg.py:62-91); the energy of
        the last local step goes to en_out[k] on the device."""
        n = self.nsites
        for i in range(n - 1):
            self.site_eigh(i)
            c = self.qr_left(i)
            self.absorb_left(c, i + 1, self.mixed_absorb(c, i + 1))
            self.env_left(i)
        for i in reversed(range(1, n)):
            self.site_eigh(i)
            c = self.qr_right(i)
            self.absorb_right(c, i - 1, self.mixed_absorb(c, i - 1))
            self.env_right(i)
        self.qr_right(0)
        en_out[k:k + 1].copy_(self.krylov_field_f64("eval0"))

    def krylov_field_f64(self, name):
        off = getattr(_lib.KrylovState, name).offset
        return self.state[off:off + 8].view(torch.float64)

    def krylov_state(self):
        raw = bytes(self.state[: _lib.C.sizeof(_lib.KrylovState)].cpu().numpy())
        return _lib.KrylovState.from_buffer_copy(raw)

    def breakdowns(self):
        return self.krylov_state().breakdowns


def warn_breakdowns(chain):
    nb = chain.breakdowns()
    if nb:
        warnings.warn(f"Lanczos iteration stopped early (beta ~= 0) in {nb} local step(s).",
                      RuntimeWarning, stacklevel=3)
