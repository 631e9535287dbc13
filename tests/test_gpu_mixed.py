"""Mixed-precision form (fixed-point BF16 digit products on tcgen05): the
tensor-core GEMM and the contractions against FP64 / the oracle, and whole sweeps
against the FP64 form. Five 8-bit digits per row-scaled value, exact integer
accumulation of digit levels 0..2 and bounded FP32 accumulation of levels 3..4
leave ~2^-39 of the row maxima: tolerances 1e-10 relative for single
contractions, stated per test for sweeps."""

import numpy as np
import pytest

from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu


def rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)


@pytest.fixture(scope="module")
def ptg():
    import pytenet_gb300 as m
    from pytenet_gb300 import _lib
    _lib.load()
    return m


def split_gemm(A, B):
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import to_dev, to_host, ptr, stream_ptr, empty
    L = _lib.load()
    M, K = A.shape
    N = B.shape[1]
    dA, dB = to_dev(A), to_dev(B)
    dC = empty((M, N))
    wsb = L.ptn_zgemm_split_bf16_workspace_bytes(M, N, K)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(L.ptn_zgemm_split_bf16(ptr(dA), K, ptr(dB), N, ptr(dC), N, M, N, K, ptr(ws), wsb,
                                      stream_ptr()))
    out = to_host(dC)
    assert L.ptn_tc_error() == 0
    return out


@pytest.mark.parametrize("mnk", [(1, 1, 1), (7, 5, 3), (128, 128, 32), (300, 257, 100),
                                 (1024, 1024, 512), (2560, 1024, 512), (512, 512, 5120)])
def test_split_bf16_gemm(ptg, mnk):
    M, N, K = mnk
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    A = orc.crandn((M, K), rng)
    B = orc.crandn((K, N), rng)
    C = split_gemm(A, B)
    ref = A @ B
    err = rel(C, ref)
    print("split gemm", mnk, err)
    assert err < 1e-10, err


@pytest.mark.parametrize("mnk", [(7, 5, 3), (1024, 2560, 512), (512, 1024, 2560),
                                 (300, 257, 3000), (2048, 1024, 1024)])
def test_persistent_gemm_equals_one_cta_per_tile(ptg, mnk):
    """PTN_TUNE_TC_PERSISTENT 1 (one CTA per SM over all (tile, K split) units) and 0
    (one CTA per unit) run the same per-unit arithmetic: bit-identical results,
    also with several units per CTA and K splits."""
    from pytenet_gb300 import _lib
    L = _lib.load()
    M, N, K = mnk
    rng = np.random.default_rng(M + 5 * N + 11 * K)
    A = orc.crandn((M, K), rng)
    B = orc.crandn((K, N), rng)
    old = L.ptn_tune_get(_lib.TUNE_TC_PERSISTENT)
    try:
        assert L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, 1) == 0
        C1 = split_gemm(A, B)
        assert L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, 0) == 0
        C0 = split_gemm(A, B)
    finally:
        L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, old)
    assert np.array_equal(C1, C0)
    assert rel(C1, A @ B) < 1e-10


def test_split_bf16_gemm_zero_rows_and_scales(ptg):
    """All-zero rows / columns (block-sparse tensors) and rows of very different
    magnitude: each row carries its own power-of-two scale."""
    rng = np.random.default_rng(99)
    A = orc.crandn((96, 70), rng)
    B = orc.crandn((70, 50), rng)
    A[5, :] = 0
    A[17:20, :] = 0
    B[:, 3] = 0
    A[30, :] *= 1e-12
    B[:, 40] *= 1e9
    C = split_gemm(A, B)
    ref = A @ B
    assert np.all(C[5] == 0) and np.all(C[:, 3] == 0)
    # fixed-point digits per row: the error of C[m, n] is bounded relative to
    # max|A[m, :]| * max|B[:, n]| * sqrt(K), whatever the magnitudes of m and n
    scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * np.sqrt(A.shape[1])
    err = np.abs(C - ref) / np.maximum(scale, 1e-300)
    assert err.max() < 1e-10, err.max()


def same_sign_case(kind, M, N, K, rng):
    """Operands whose real GEMM (plain A times embedded B) has every product of one
    sign: the worst case for FP32 accumulation of the digit levels."""
    if kind == "constant":
        # identical digits in every entry: every level sum grows linearly in K
        A = np.full((M, K), 0.7123456789 + 0.4567891234j)
        B = np.full((K, N), 0.9876543211 + 0.0j)
    elif kind == "positive":
        A = rng.uniform(0.5, 1.0, (M, K)) + 1j * rng.uniform(0.5, 1.0, (M, K))
        B = rng.uniform(0.5, 1.0, (K, N)) + 0j
    elif kind == "psd-env":
        # a positive-semidefinite Hermitian environment block X X^H (positive X)
        # against a non-negative site tensor: the shape of an environment step
        X = rng.uniform(0.0, 1.0, (max(M, K), 8))
        A = (X @ X.T)[:M, :K] + 0j
        B = rng.uniform(0.0, 1.0, (K, N)) + 0j
    elif kind == "dominant":
        # one dominant element per row next to small same-sign ones
        A = rng.uniform(0.0, 1e-3, (M, K)) + 0j
        A[np.arange(M), rng.integers(0, K, M)] = 1.0
        B = rng.uniform(0.5, 1.0, (K, N)) + 0j
    else:
        raise ValueError(kind)
    return A, B


@pytest.mark.parametrize("kind", ["constant", "positive", "psd-env", "dominant"])
@pytest.mark.parametrize("mnk", [(256, 192, 1024), (200, 160, 5120), (1024, 512, 5120)])
def test_split_bf16_gemm_same_sign(ptg, kind, mnk):
    """Exactness does not depend on random signs: with every digit product of one
    sign (the worst case for the level sums) at K = 2048 and 10240 reals, and at
    the environment shapes of D = 1024 (K = 5120 complex), the error stays below
    1e-10 max|A| max|B| K."""
    M, N, K = mnk
    rng = np.random.default_rng(M + N + K)
    A, B = same_sign_case(kind, M, N, K, rng)
    C = split_gemm(A, B)
    ref = A @ B
    scale = np.abs(A).max() * np.abs(B).max() * K
    err = np.abs(C - ref).max() / scale
    # and element by element against the row and column maxima
    rs = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * K
    err_el = (np.abs(C - ref) / np.maximum(rs, 1e-300)).max()
    print("same-sign gemm", kind, mnk, err, err_el)
    assert err < 1e-10, err
    assert err_el < 1e-10, err_el


@pytest.mark.parametrize("dims", [(1, 2, 2, 1, 5), (16, 2, 32, 5, 5), (64, 2, 64, 5, 5),
                                  (130, 2, 97, 4, 5), (256, 2, 256, 5, 5),
                                  (512, 2, 512, 5, 5)])
def test_mixed_contractions(ptg, dims):
    """Every contraction of the mixed form against the oracle, up to the D = 512
    bulk shapes of the L = 64 chain (Dl = Dr = 512, chi = 5)."""
    Dl, d, Dr, cl, cr = dims
    rng = np.random.default_rng(11 + sum(dims))
    a = orc.crandn((Dl, d, Dr), rng)
    w = rng.normal(size=(cl, d, d, cr))
    w[np.abs(w) < 0.7] = 0.0
    l = orc.crandn((Dl, cl, Dl), rng)
    r = orc.crandn((Dr, cr, Dr), rng)
    tol = 1e-10
    assert rel(ptg.apply_local_hamiltonian(a, w, l, r, precision="mixed"),
               orc.apply_local_hamiltonian(a, w, l, r)) < tol
    assert rel(ptg.contraction_operator_step_left(a, a, w, l, precision="mixed"),
               orc.env_step_left(a, a, w, l)) < tol
    assert rel(ptg.contraction_operator_step_right(a, a, w, r, precision="mixed"),
               orc.env_step_right(a, a, w, r)) < tol
    c = orc.crandn((Dl, Dr), rng)
    lb = orc.crandn((Dl, cr, Dl), rng)
    assert rel(ptg.apply_local_bond_contraction(c, lb, r, precision="mixed"),
               orc.apply_local_bond_contraction(c, lb, r)) < tol


def tc_launches(fn):
    """Run fn and count the tensor-core GEMM launches it made (kind 1 of the
    library's profiling hooks)."""
    import ctypes
    import torch
    from pytenet_gb300 import _lib
    L = _lib.load()
    torch.cuda.synchronize()
    L.ptn_prof_start(1 << 1)
    out = fn()
    torch.cuda.synchronize()
    L.ptn_prof_stop()
    tot, fl, by, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
    _lib.check(L.ptn_prof_read(1, ctypes.byref(tot), ctypes.byref(fl), ctypes.byref(by),
                               ctypes.byref(n)))
    return out, n.value


def test_mixed_tdvp_tracks_fp64(ptg):
    """L=20, D=128 real time, 3 steps: mixed vs FP64 energy and fidelity. Bonds of
    32 and more run on the tensor cores (the mixed form keeps smaller local
    problems in FP64)."""
    rng = np.random.default_rng(3)
    L, D = 20, 128
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    p64 = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
    p64.a = [x.copy() for x in psi.a]
    pmx = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
    pmx.a = [x.copy() for x in psi.a]
    ptg.tdvp_singlesite(h, p64, 0.05j, 3, numiter_lanczos=8, precision="fp64")
    _, ntc = tc_launches(lambda: ptg.tdvp_singlesite(h, pmx, 0.05j, 3, numiter_lanczos=8,
                                                     precision="mixed"))
    assert ntc > 100
    e64 = orc.mpo_average(p64, h).real
    emx = orc.mpo_average(pmx, h).real
    ov = orc.mps_vdot(p64, pmx)
    n64, nmx = orc.mps_vdot(p64, p64).real, orc.mps_vdot(pmx, pmx).real
    infid = 1 - abs(ov) ** 2 / (n64 * nmx)
    print("energy rel err", abs(emx - e64) / abs(e64), "infidelity", infid,
          "norm drift", abs(np.sqrt(nmx) - np.sqrt(n64)), "tc launches", ntc)
    # a random state's energy is close to zero, so the energy error is also
    # bounded against the chain's energy scale L J; targets of the mixed form:
    # relative energy error 1e-8, infidelity 1e-9
    assert abs(emx - e64) < 1e-8 * abs(e64) and abs(emx - e64) < 1e-11 * L
    assert infid < 1e-12


def test_mixed_dmrg_energy(ptg):
    rng = np.random.default_rng(4)
    L = 16
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 1.0, 0.0)
    psi = ptg.MPS.construct_random(L, h.qsite, 0, max_vdim=128, dtype="complex", rng=rng)
    p2 = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
    p2.a = [x.copy() for x in psi.a]
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        e64 = ptg.dmrg_singlesite(h, psi, 3, numiter_lanczos=20, precision="fp64")
        emx, ntc = tc_launches(lambda: ptg.dmrg_singlesite(h, p2, 3, numiter_lanczos=20,
                                                           precision="mixed"))
    print("dmrg energies", e64[-1], emx[-1], "tc launches", ntc)
    assert ntc > 100
    # the Ritz value is first-order in the ~1e-11 relative contraction error
    assert abs(emx[-1] - e64[-1]) < 1e-10 * abs(e64[-1])
