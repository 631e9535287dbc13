"""Block-sparse contractions: with quantum numbers every tensor holds zero blocks
(pytenet/block_sparse_util.py:47-64), and after the first block QR every bond is
ordered by quantum number, so the FP64 GEMMs skip the K slabs whose A or B part of a
tile is zero, and the tensor-core digit GEMMs of the mixed form skip the K blocks
whose A or B tile is zero (flags from the digit conversion). Checked against the
oracle on a U(1)-conserving XXZ run (the reference's quantum-number test setup,
test/test_tdvp.py:26-49, at larger bonds), the skipping digit GEMM bit for bit
against the one that multiplies every block, and timed against a dense state with
the same bond dimensions."""

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


def test_digit_gemm_skips_zero_tiles_exactly():
    """Operands with quantum-number-like zero blocks: the digit GEMM with zero-tile
    skipping (PTN_TUNE_TC_SKIP_ZERO 1: the K blocks where the A or the B tile is
    zero are not multiplied) gives the same bits as the persistent and the
    one-CTA-per-unit kernels without it."""
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import to_dev, to_host, ptr, stream_ptr, empty
    L = _lib.load()
    rng = np.random.default_rng(43)
    M, N, K = 640, 500, 700
    A = np.zeros((M, K), complex)
    B = np.zeros((K, N), complex)
    # sector boundaries not aligned with the 128 x 16 / 48 x 16 tiles
    rs, ks, cs = [0, 200, 390, 640], [0, 150, 420, 700], [0, 170, 333, 500]
    for j in range(3):
        A[rs[j]:rs[j + 1], ks[j]:ks[j + 1]] = orc.crandn((rs[j + 1] - rs[j], ks[j + 1] - ks[j]), rng)
        B[ks[j]:ks[j + 1], cs[j]:cs[j + 1]] = orc.crandn((ks[j + 1] - ks[j], cs[j + 1] - cs[j]), rng)
    out = {}
    old = (L.ptn_tune_get(_lib.TUNE_TC_PERSISTENT), L.ptn_tune_get(_lib.TUNE_TC_SKIP_ZERO))
    try:
        for pers, skip in ((1, 1), (1, 0), (0, 0)):
            assert L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, pers) == 0
            assert L.ptn_tune_set(_lib.TUNE_TC_SKIP_ZERO, skip) == 0
            dA, dB, dC = to_dev(A), to_dev(B), empty((M, N))
            wsb = L.ptn_zgemm_split_bf16_workspace_bytes(M, N, K)
            ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
            _lib.check(L.ptn_zgemm_split_bf16(ptr(dA), K, ptr(dB), N, ptr(dC), N, M, N, K, ptr(ws),
                                              wsb, stream_ptr()))
            out[(pers, skip)] = to_host(dC)
            assert L.ptn_tc_error() == 0
    finally:
        L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, old[0])
        L.ptn_tune_set(_lib.TUNE_TC_SKIP_ZERO, old[1])
    assert np.array_equal(out[(1, 1)], out[(1, 0)])
    assert np.array_equal(out[(1, 1)], out[(0, 0)])
    ref = A @ B
    assert np.linalg.norm(out[(1, 1)] - ref) < 1e-10 * np.linalg.norm(ref)


def test_blocksparse_mixed_tdvp_tracks_fp64():
    """U(1) XXZ, mixed form (digit GEMMs skipping zero tiles) against the FP64 form
    on the same state: energy within 1e-10 relative, infidelity below 1e-10, same
    bond quantum numbers; the same mixed step without skipping gives the same
    tensors, and one step of each is timed."""
    import torch
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    L_ = _lib.load()
    rng = np.random.default_rng(44)
    L, D, m = 20, 256, 8
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    psi = u1_state(ptg, h, L, D, rng)
    psi.orthonormalize(mode="left")
    res, times = {}, {}
    old = L_.ptn_tune_get(_lib.TUNE_TC_SKIP_ZERO)
    try:
        for form, pers in (("fp64", 1), ("mixed", 0), ("mixed", 1)):
            assert L_.ptn_tune_set(_lib.TUNE_TC_SKIP_ZERO, pers) == 0
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                for k in range(2):   # warm-up, then timed
                    p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
                    p.a = [x.copy() for x in psi.a]
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    ptg.tdvp_singlesite(h, p, 0.05j, 1, numiter_lanczos=m, precision=form)
                    torch.cuda.synchronize()
                    times[(form, pers)] = time.perf_counter() - t0
            res[(form, pers)] = p
    finally:
        L_.ptn_tune_set(_lib.TUNE_TC_SKIP_ZERO, old)
    p64, pmx = res[("fp64", 1)], res[("mixed", 1)]
    ov = orc.mps_vdot(p64, pmx)
    infid = 1 - abs(ov) ** 2 / (orc.mps_vdot(p64, p64).real * orc.mps_vdot(pmx, pmx).real)
    e64, emx = orc.mpo_average(p64, h).real, orc.mpo_average(pmx, h).real
    for qa, qb in zip(p64.qbonds, pmx.qbonds):
        assert np.array_equal(qa, qb)
    print(f"U(1) XXZ L={L}, bonds <= {D}, mixed vs fp64: energy {abs(emx - e64) / abs(e64):.1e}, "
          f"infidelity {infid:.1e}; one step: fp64 {times[('fp64', 1)]:.3f} s, mixed dense "
          f"{times[('mixed', 0)]:.3f} s, mixed skipping zero tiles {times[('mixed', 1)]:.3f} s")
    assert abs(emx - e64) < 1e-10 * abs(e64) and infid < 1e-10
    assert np.allclose(res[("mixed", 0)].a[L // 2], pmx.a[L // 2], rtol=0, atol=1e-12)
