"""The fused Lanczos step (one cooperative launch per iteration: dot, three-term
update, norm, breakdown test and scaling with two grid barriers) against the
three-launch step, on the same inputs (pytenet/krylov.py:12-57). Summation orders
differ, so results agree to rounding, not bit for bit."""

import warnings

import numpy as np
import pytest

from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu


def _run(ptg, fused, graph):
    from pytenet_gb300 import _lib
    L = _lib.load()
    old = L.ptn_tune_get(_lib.TUNE_KRYLOV_FUSED)
    _lib.check(L.ptn_tune_set(_lib.TUNE_KRYLOV_FUSED, 1 if fused else 0))
    try:
        rng = np.random.default_rng(31)
        # the fused step serves vectors of at least 2^18 entries: the middle sites of
        # L = 20 at D = 512 (2 * 512^2 entries); smaller ones take three launches
        Lx, D = 20, 512
        h = ptg.heisenberg_xxz_1d_mpo(Lx, 1.0, 0.8, -0.1)
        h.zero_qnumbers()
        b = [min(2 ** min(i, Lx - i), D) for i in range(Lx + 1)]
        psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
        psi.orthonormalize(mode="left")
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            run = ptg.TDVPRun(h, psi, numiter_lanczos=8, precision="mixed", graph=graph)
            for _ in range(2):
                run.step(0.05j)
        run.download()
        return psi, run.chain.krylov_state()
    finally:
        L.ptn_tune_set(_lib.TUNE_KRYLOV_FUSED, old)


def test_fused_lanczos_matches_three_launch_step():
    import pytenet_gb300 as ptg
    p3, s3 = _run(ptg, fused=False, graph=False)
    pf, sf = _run(ptg, fused=True, graph=False)
    pg, sg = _run(ptg, fused=True, graph=True)
    assert sf.status == 0 and sg.status == 0
    # same depths and breakdowns (edge sites exhaust their Krylov space)
    assert sf.iters_total == s3.iters_total and sf.breakdowns == s3.breakdowns
    # the mixed form's contractions carry ~1e-11 relative error that depends on the
    # digits of their input, so the rounding-level difference of the two reduction
    # orders perturbs the states at that level: compared by fidelity and energy
    h = ptg.heisenberg_xxz_1d_mpo(20, 1.0, 0.8, -0.1)
    ov = orc.mps_vdot(p3, pf)
    infid = 1 - abs(ov) ** 2 / (orc.mps_vdot(p3, p3).real * orc.mps_vdot(pf, pf).real)
    e3, ef = orc.mpo_average(p3, h).real, orc.mpo_average(pf, h).real
    assert infid < 1e-12 and abs(e3 - ef) < 1e-10 * 20
    for y, z in zip(pf.a, pg.a):
        assert np.array_equal(y, z)   # graph replay of the cooperative launch == eager
    print("fused vs three-launch: infidelity", infid, "energy", abs(e3 - ef))


def test_fused_lanczos_breakdown_like_reference():
    """A Hermitian operator of rank 5 on vectors of 2^18 entries (the fused step):
    the Krylov space is exhausted after 5 steps and the run stops there, as
    lanczos_iteration does (krylov.py:44-50)."""
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    L = _lib.load()
    assert L.ptn_tune_get(_lib.TUNE_KRYLOV_FUSED) == 1
    rng = np.random.default_rng(32)
    n = 1 << 18
    u = np.linalg.qr(orc.crandn((n, 5), rng))[0]
    lam = np.array([1.0, -2.0, 3.0, 0.5, -1.5])

    def op(x):
        return u @ (lam * (u.conj().T @ x))

    v0 = orc.crandn(n, rng)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        a1, b1, V1 = ptg.lanczos_iteration(op, v0, 12)
        a2, b2, V2 = orc.lanczos_iteration(op, v0, 12)
    assert len(a1) == len(a2) and len(b1) == len(b2)
    assert np.allclose(a1, a2, rtol=0, atol=1e-12) and np.allclose(b1, b2, rtol=0, atol=1e-12)
