"""Host-side logic of pytenet_gb300 (no GPU): the C ABI library loads and exports
every declared symbol, integer quantum-number plans match the reference, the
input generators reproduce the reference's draws and operators."""

import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden, golden_mps, golden_mpo
from oracle import ptn_oracle as orc


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "pytenet_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ptn_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    import ctypes
    from pytenet_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    from pytenet_gb300 import _lib
    assert set(_lib.exported_names()) == set(syms)
    L = _lib.load(path)
    assert L.ptn_abi_version() == _lib.ABI_VERSION == 3
    assert b"sm_103a" in L.ptn_version()


def test_workspace_queries_need_no_gpu():
    from pytenet_gb300 import _lib
    L = _lib.load()
    assert L.ptn_krylov_state_bytes() >= ctypes_sizeof_state()
    assert L.ptn_qr_workspace_bytes(1024, 512) > 1024 * 512 * 16
    assert L.ptn_heff_workspace_bytes(64, 2, 64, 5, 5, 0) >= 2 * 64 * 10 * 64 * 16


def ctypes_sizeof_state():
    import ctypes
    from pytenet_gb300 import _lib
    return ctypes.sizeof(_lib.KrylovState)


def test_qr_plans_match_reference_bookkeeping():
    from pytenet_gb300.qnumber import qr_plan
    g = load_golden("block_qr.npz")
    for k in range(int(g["ncases"])):
        plan = qr_plan(g[f"q0_{k}"], g[f"q1_{k}"])
        assert np.array_equal(plan.qinterm, g[f"qi{k}"])
        assert plan.K == g[f"q{k}"].shape[1]


def test_random_mps_draw_order():
    import pytenet_gb300 as ptg
    g = load_golden("mps_random.npz")
    ref = golden_mps(g, "r_")
    psi = ptg.MPS(ref.qsite, ref.qbonds, fill="random", rng=np.random.default_rng(1009))
    for x, y in zip(psi.a, ref.a):
        assert np.array_equal(x, y)
    ref = golden_mps(g, "c_")
    psi = ptg.MPS.construct_random(7, [1, -1], 1, max_vdim=6, dtype="complex",
                                   rng=np.random.default_rng(1010))
    for q, qr in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(q, qr)
    for x, y in zip(psi.a, ref.a):
        assert np.array_equal(x, y)
    ref = golden_mps(g, "d_")
    psi = ptg.MPS.construct_random(6, [1, -1], 0, max_vdim=5, dtype="real",
                                   rng=np.random.default_rng(1011))
    for x, y in zip(psi.a, ref.a):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("L", [2, 3, 4, 5, 6])
def test_hamiltonians_equal_reference_operators(L):
    import pytenet_gb300 as ptg
    g = load_golden("mpos.npz")
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.3, 0.7, -0.2)
    # the reference's bond dimensions: 4 next to the chain ends, 5 in the bulk
    assert list(h.bond_dims) == [1] + [4] + [5] * (L - 3) + [4] * (L > 2) + [1]
    assert np.allclose(h.to_matrix(), g[f"xxz{L}_mat"], rtol=0, atol=1e-14)
    assert np.allclose(orc.mpo_to_matrix(h), g[f"xxz{L}_mat"], rtol=0, atol=1e-14)
    for i, w in enumerate(h.a):
        assert orc.is_qsparse(w, (h.qbonds[i], h.qsite, -h.qsite, -h.qbonds[i + 1]))
    s = ptg.ising_1d_mpo(L, 1.0, 0.15, 0.8)
    assert np.allclose(s.to_matrix(), g[f"ising{L}_mat"], rtol=0, atol=1e-14)


def test_to_vector_matches_oracle():
    import pytenet_gb300 as ptg
    g = load_golden("tdvp_readme.npz")
    ref = golden_mps(g, "p1_")
    psi = ptg.MPS(ref.qsite, ref.qbonds, fill="postpone")
    psi.a = [x.copy() for x in ref.a]
    assert np.allclose(psi.to_vector(), g["v1"], atol=1e-14)
    assert np.allclose(psi.as_vector(), orc.mps_to_vector(ref), atol=1e-14)


def test_product_package_does_not_import_oracle():
    pkg = os.path.join(ROOT, "pytenet_gb300")
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            src = open(os.path.join(pkg, f)).read()
            assert "oracle" not in src.replace("the oracle", ""), f


def test_no_gpu_means_loud_failure():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import pytenet_gb300 as ptg
    h = ptg.heisenberg_xxz_1d_mpo(4, 1.0, 0.8, -0.1)
    psi = ptg.MPS(h.qsite, [[0], [0, 0], [0, 0], [0, 0], [0]], fill="random",
                  rng=np.random.default_rng(0))
    with pytest.raises(RuntimeError):
        ptg.tdvp_singlesite(h, psi, 0.1j, 1, numiter_lanczos=3)


def test_c_abi_argument_errors_without_gpu():
    """Shape / argument checks of the C ABI come before any device work and map to
    PTN_BAD_SHAPE with a message (the reference raises AssertionError there)."""
    from pytenet_gb300 import _lib
    L = _lib.load()
    C = _lib.C
    null = None
    # empty matrix
    assert L.ptn_qr(null, 0, 4, null, 4, null, 4, null, 0, null) == _lib.PTN_BAD_SHAPE
    assert b"empty" in L.ptn_last_error()
    # ragged / zero dimensions of the effective Hamiltonian
    assert L.ptn_heff_apply(null, null, null, null, null, 0, 2, 4, 5, 5, 0, null, 0,
                            null) == _lib.PTN_BAD_SHAPE
    assert L.ptn_env_step_left(null, null, null, null, null, 4, 2, 0, 5, 5, 0, null, 0,
                               null) == _lib.PTN_BAD_SHAPE
    # unknown transposition code of the GEMM
    assert L.ptn_zgemm(b"X", b"N", 4, 4, 4, _lib.cval(1), null, 4, 0, null, 4, 0, _lib.cval(0),
                       null, 4, 0, 1, null, 0, null) == _lib.PTN_BAD_SHAPE
    assert b"bad op" in L.ptn_last_error()
    # Python layer: shape errors are AssertionErrors, like the reference's
    err = _lib.PtnShapeError(_lib.PTN_BAD_SHAPE, "x")
    assert isinstance(err, AssertionError)


def test_retained_bond_indices_matches_oracle():
    """Truncation rule of the two-site splits (pytenet/bond_ops.py:23-38), including
    an all-zero spectrum and exact zeros."""
    from pytenet_gb300.bond_ops import retained_bond_indices
    rng = np.random.default_rng(5)
    cases = [np.zeros(4), np.array([3.0, 0.0, 0.0]), np.array([1.0])]
    for _ in range(100):
        cases.append(np.sort(rng.exponential(size=rng.integers(1, 30)))[::-1] ** 4)
    for s in cases:
        for tol in (0.0, 1e-14, 1e-10, 1e-6, 1e-2):
            assert np.array_equal(retained_bond_indices(s, tol), orc.retained_bond_indices(s.copy(), tol))


def test_merge_mpo_pair_matches_oracle():
    from pytenet_gb300.twosite import merge_mpo_pair
    rng = np.random.default_rng(6)
    w0 = rng.normal(size=(3, 2, 2, 4))
    w1 = rng.normal(size=(4, 2, 2, 5))
    assert np.allclose(merge_mpo_pair(w0, w1), orc._mpo_merge_pair(w0, w1), rtol=0, atol=1e-14)


def test_density_compression_column_order_matches_block_sparse_eigh():
    """compression._eigh_order puts the block SVD's columns (sorted quantum-number
    blocks, values descending) into block_sparse_eigh's order (blocks in the
    iteration order of the Python set of the row quantum numbers, eigenvalues
    ascending; pytenet/block_sparse_util.py:183-241). Checked on a Hermitian
    positive semidefinite block-sparse matrix with a NumPy SVD per plan block:
    the permuted singular values equal the oracle's |eigenvalues| and the permuted
    quantum numbers its bond quantum numbers, position by position."""
    from pytenet_gb300.compression import _eigh_order
    from pytenet_gb300.qnumber import qr_plan
    rng = np.random.default_rng(7)
    q = rng.choice([-3, -1, 0, 1, 2, 5], size=40)
    b = orc.crandn((40, 40), rng)
    b[q[:, None] != q[None, :]] = 0
    rho = b @ b.conj().T                       # block-diagonal in q, PSD
    plan = qr_plan(q, q)
    s = np.zeros(plan.K)
    for rows, cols, k0, kb in plan.blocks:
        s[k0:k0 + kb] = np.linalg.svd(rho[np.ix_(rows, cols)], compute_uv=False)
    perm = _eigh_order(plan, q)
    u, ev, qe = orc.block_sparse_eigh(rho, q)
    assert sorted(perm.tolist()) == list(range(plan.K))
    assert np.array_equal(plan.qinterm[perm], qe)
    assert np.allclose(s[perm], np.abs(ev), rtol=0, atol=1e-10 * np.abs(ev).max())


def test_is_qsparse_without_constraints_and_with_violations():
    """is_qsparse (pytenet/block_sparse_util.py:47-53): nothing is constrained when
    every quantum-number sum is zero (any tensor passes, without looking at it);
    with quantum numbers a non-zero entry at a non-zero sum is detected."""
    from pytenet_gb300.qnumber import is_qsparse, enforce_qsparsity
    rng = np.random.default_rng(8)
    a = orc.crandn((4, 2, 5), rng)
    assert is_qsparse(a, [np.zeros(4, int), np.zeros(2, int), np.zeros(5, int)])
    qn = [np.array([0, 1, -1, 2]), np.array([1, -1]), -np.array([1, 0, -1, 2, 3])]
    assert not is_qsparse(a, qn) and not orc.is_qsparse(a, qn)
    enforce_qsparsity(a, qn)
    assert is_qsparse(a, qn) and orc.is_qsparse(a, qn)
