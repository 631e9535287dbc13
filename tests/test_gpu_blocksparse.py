"""Block-sparse contractions: with quantum numbers every tensor holds zero blocks
(pytenet/block_sparse_util.py:47-64), and after the first block QR every bond is
ordered by quantum number, so the FP64 GEMMs skip the K slabs whose A or B part of a
tile is zero. Checked against the oracle on a U(1)-conserving XXZ run (the reference's
quantum-number test setup, test/test_tdvp.py:26-49, at larger bonds), and timed
against a dense state with the same bond dimensions."""

import time
import warnings

import numpy as np
import pytest

from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu


def u1_state(ptg, h, L, D, rng):
    """Random spin-sector MPS (total 2 Sz = 0) with bonds of at most D entries,
    the quantum numbers of each bond drawn from the values reachable from both
    chain ends."""
    qb = [np.array([0])]
    for i in range(1, L):
        reach = min(i, L - i)
        vals = np.arange(-reach, reach + 1, 2)
        n = min(2 ** reach, D)
        qb.append(np.sort(rng.choice(vals, size=n, replace=True)))
    qb.append(np.array([0]))
    return ptg.MPS(h.qsite, qb, fill="random", rng=rng)


def test_blocksparse_tdvp_matches_oracle():
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    _lib.load()
    rng = np.random.default_rng(41)
    L, D, steps, m = 16, 128, 2, 8
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    psi = u1_state(ptg, h, L, D, rng)
    psi.orthonormalize(mode="left")
    bonds = [len(q) for q in psi.qbonds]
    ref = orc.OMPS(psi.qsite, psi.qbonds, [x.copy() for x in psi.a])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        orc.tdvp_singlesite(h, ref, 0.05j, steps, numiter_lanczos=m)
        p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
        p.a = [x.copy() for x in psi.a]
        ptg.tdvp_singlesite(h, p, 0.05j, steps, numiter_lanczos=m)
    # same result as the oracle
    ov = orc.mps_vdot(ref, p)
    infid = 1 - abs(ov) ** 2 / (orc.mps_vdot(ref, ref).real * orc.mps_vdot(p, p).real)
    e, er = orc.mpo_average(p, h).real, orc.mpo_average(ref, h).real
    assert infid < 1e-12 and abs(e - er) < 1e-10 * max(1.0, abs(er))
    for qa, qr_ in zip(p.qbonds, ref.qbonds):
        assert np.array_equal(qa, qr_)
    print(f"U(1) XXZ L={L}, bonds up to {max(bonds)}: infidelity vs oracle {infid:.1e}")


def _timed_tdvp(ptg, h, psi, steps, m):
    import torch
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for k in range(2):   # once to warm up, once timed
            p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
            p.a = [x.copy() for x in psi.a]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ptg.tdvp_singlesite(h, p, 0.05j, steps, numiter_lanczos=m)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
    return t


def test_blocksparse_saves_time_at_larger_bonds():
    """L = 24 with bonds up to 256: the U(1) state against a dense state with the
    same bond dimensions (zero quantum numbers), one FP64 time step each."""
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    _lib.load()
    rng = np.random.default_rng(42)
    L, D, m = 24, 256, 8
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    psi = u1_state(ptg, h, L, D, rng)
    psi.orthonormalize(mode="left")
    bonds = [len(q) for q in psi.qbonds]
    t_sparse = _timed_tdvp(ptg, h, psi, 1, m)
    hd = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    hd.zero_qnumbers()
    pd = ptg.MPS(hd.qsite, [b * [0] for b in bonds], fill="random", rng=rng)
    pd.orthonormalize(mode="left")
    t_dense = _timed_tdvp(ptg, hd, pd, 1, m)
    sectors = len(np.unique(psi.qbonds[L // 2]))
    print(f"U(1) XXZ L={L}, bonds up to {max(bonds)} ({sectors} sectors mid-chain): "
          f"block-sparse {t_sparse:.3f} s, dense with the same bonds {t_dense:.3f} s "
          f"({t_dense / t_sparse:.2f}x)")
    assert t_sparse < t_dense
