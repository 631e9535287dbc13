"""Parity of the GPU engine (through the C ABI) with the CPU oracle and with the
reference's golden outputs. Plain complex128 form: tolerances as stated per test
(1e-12 relative for single contractions, 1e-10 for whole sweeps)."""

import copy
import warnings

import numpy as np
import pytest

from conftest import load_golden, golden_mps, golden_mpo
from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)


@pytest.fixture(scope="module")
def ptg():
    import pytenet_gb300 as m
    from pytenet_gb300 import _lib
    _lib.load()
    return m


def as_ptg_mps(ptg, o):
    psi = ptg.MPS(o.qsite, o.qbonds, fill="postpone")
    psi.a = [np.array(x, dtype=np.complex128) for x in o.a]
    psi.qbonds = [np.array(q) for q in o.qbonds]
    return psi


# --------------------------------------------------------------------- contractions

def test_chain_ops_golden(ptg):
    g = load_golden("chain_ops.npz")
    assert rel(ptg.apply_local_hamiltonian(g["a"], g["w"], g["l"], g["r"]), g["heff"]) < RTOL
    assert rel(ptg.apply_local_hamiltonian(g["a"], g["wc"], g["l"], g["r"]), g["heff_c"]) < RTOL
    assert rel(ptg.apply_local_bond_contraction(g["c"], g["lb"], g["r"]), g["bond"]) < RTOL
    assert rel(ptg.contraction_operator_step_left(g["a"], g["b"], g["w"], g["l"]), g["env_left"]) < RTOL
    assert rel(ptg.contraction_operator_step_right(g["a"], g["b"], g["w"], g["r"]), g["env_right"]) < RTOL
    assert rel(ptg.contraction_operator_step_left(g["a"], g["a"], g["wc"], g["l"]), g["env_left_aa"]) < RTOL
    assert rel(ptg.contraction_operator_step_right(g["a"], g["a"], g["wc"], g["r"]), g["env_right_aa"]) < RTOL


@pytest.mark.parametrize("dims", [(1, 2, 2, 1, 5), (16, 2, 32, 5, 5), (64, 2, 64, 5, 5),
                                  (130, 2, 97, 4, 5), (256, 2, 256, 5, 5), (33, 3, 20, 7, 3)])
def test_contractions_random(ptg, dims):
    Dl, d, Dr, cl, cr = dims
    rng = np.random.default_rng(sum(dims))
    a = orc.crandn((Dl, d, Dr), rng)
    w = rng.normal(size=(cl, d, d, cr))
    w[np.abs(w) < 0.7] = 0.0    # MPO-like sparsity
    l = orc.crandn((Dl, cl, Dl), rng)
    r = orc.crandn((Dr, cr, Dr), rng)
    assert rel(ptg.apply_local_hamiltonian(a, w, l, r), orc.apply_local_hamiltonian(a, w, l, r)) < RTOL
    assert rel(ptg.contraction_operator_step_left(a, a, w, l), orc.env_step_left(a, a, w, l)) < RTOL
    assert rel(ptg.contraction_operator_step_right(a, a, w, r), orc.env_step_right(a, a, w, r)) < RTOL
    c = orc.crandn((Dl, Dr), rng)
    lb = orc.crandn((Dl, cr, Dl), rng)
    assert rel(ptg.apply_local_bond_contraction(c, lb, r), orc.apply_local_bond_contraction(c, lb, r)) < RTOL


@pytest.mark.parametrize("opa", "NTCH")
@pytest.mark.parametrize("opb", "NTCH")
def test_zgemm_ops(ptg, opa, opb):
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import to_dev, to_host, ptr, stream_ptr
    rng = np.random.default_rng(ord(opa) * 7 + ord(opb))
    for (M, N, K) in [(7, 5, 3), (64, 64, 16), (100, 70, 300), (33, 129, 2000)]:
        A = orc.crandn((M, K) if opa in "NC" else (K, M), rng)
        B = orc.crandn((K, N) if opb in "NC" else (N, K), rng)
        f = {"N": lambda x: x, "T": lambda x: x.T, "C": np.conj, "H": lambda x: x.conj().T}
        ref = 0.5j * (f[opa](A) @ f[opb](B))
        C0 = orc.crandn((M, N), rng)
        ref = ref + (1 - 1j) * C0
        dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0)
        L = _lib.load()
        wsb = L.ptn_zgemm_workspace_bytes(M, N, K, 1)
        ws = torch.empty(max(wsb, 256), dtype=torch.uint8, device="cuda")
        _lib.check(L.ptn_zgemm(opa.encode(), opb.encode(), M, N, K, _lib.cval(0.5j), ptr(dA),
                               A.shape[1], 0, ptr(dB), B.shape[1], 0, _lib.cval(1 - 1j), ptr(dC), N,
                               0, 1, ptr(ws), wsb, stream_ptr()))
        assert rel(to_host(dC), ref) < RTOL


# ----------------------------------------------------------------------------- QR

@pytest.mark.parametrize("mn", [(1, 1), (2, 1), (1, 3), (5, 3), (40, 12), (12, 40), (64, 64),
                                (300, 150), (1024, 512), (77, 77)])
def test_qr_matches_lapack_convention(ptg, mn):
    m, n = mn
    rng = np.random.default_rng(m * 1000 + n)
    a = orc.crandn((m, n), rng)
    q, r, qi = ptg.block_sparse_qr(a, np.zeros(m, int), np.zeros(n, int))
    qr_, rr_ = np.linalg.qr(a, mode="reduced")
    # same Householder convention -> same factors, signs included
    assert np.allclose(q, qr_, rtol=0, atol=1e-11)
    assert np.allclose(r, rr_, rtol=0, atol=1e-11 * max(1, np.abs(rr_).max()))
    assert np.allclose(q @ r, a, atol=1e-12 * np.sqrt(m * n))


def test_qr_rank_deficient_and_real_input(ptg):
    rng = np.random.default_rng(5)
    a = orc.crandn((64, 32), rng)
    a[:, 20:] = 0
    a[:, 5] = 0
    q, r, _ = ptg.block_sparse_qr(a, np.zeros(64, int), np.zeros(32, int))
    qr_, rr_ = np.linalg.qr(a, mode="reduced")
    assert np.allclose(q, qr_, atol=1e-12) and np.allclose(r, rr_, atol=1e-12)
    b = rng.normal(size=(30, 10)).astype(complex)
    q, r, _ = ptg.block_sparse_qr(b, np.zeros(30, int), np.zeros(10, int))
    qr_, rr_ = np.linalg.qr(b, mode="reduced")
    assert np.allclose(q, qr_, atol=1e-12) and np.allclose(r, rr_, atol=1e-12)


@pytest.mark.parametrize("form", [(0, 0), (0, 1), (0, 2), (0, 3), (5, 0), (5, 1)])
def test_qr_kernel_forms_agree_with_lapack(ptg, form):
    """Every pairing of the block-update kernels (PTN_TUNE_LARFB_TILE 0: register-
    tiled, 5: the earlier three-pass form) and of the panel kernels
    (PTN_TUNE_QR_PANEL 0 .. 3) gives numpy.linalg.qr's factors, including on
    rank-deficient input and on a last panel narrower than 16 columns."""
    from pytenet_gb300 import _lib
    L = _lib.load()
    old = (L.ptn_tune_get(_lib.TUNE_LARFB_TILE), L.ptn_tune_get(_lib.TUNE_QR_PANEL))
    try:
        assert L.ptn_tune_set(_lib.TUNE_LARFB_TILE, form[0]) == 0
        assert L.ptn_tune_set(_lib.TUNE_QR_PANEL, form[1]) == 0
        rng = np.random.default_rng(77 + form[0] + 10 * form[1])
        cases = [orc.crandn((1024, 512), rng), orc.crandn((2048, 1000), rng),
                 orc.crandn((300, 150), rng), orc.crandn((40, 90), rng)]
        a = orc.crandn((256, 100), rng)
        a[:, 60:] = 0
        a[:, 7] = 0
        a[100:, :] = 0
        cases.append(a)
        for a in cases:
            m, n = a.shape
            q, r, _ = ptg.block_sparse_qr(a, np.zeros(m, int), np.zeros(n, int))
            qr_, rr_ = np.linalg.qr(a, mode="reduced")
            assert np.allclose(q, qr_, rtol=0, atol=1e-11), (m, n)
            assert np.allclose(r, rr_, rtol=0, atol=1e-11 * max(1, np.abs(rr_).max())), (m, n)
    finally:
        L.ptn_tune_set(_lib.TUNE_LARFB_TILE, old[0])
        L.ptn_tune_set(_lib.TUNE_QR_PANEL, old[1])


def test_block_sparse_qr_golden(ptg):
    g = load_golden("block_qr.npz")
    for k in range(int(g["ncases"])):
        a, q0, q1 = g[f"a{k}"], g[f"q0_{k}"], g[f"q1_{k}"]
        q, r, qi = ptg.block_sparse_qr(a, q0, q1)
        assert np.array_equal(qi, g[f"qi{k}"])                  # integer bookkeeping: exact
        assert q.shape == g[f"q{k}"].shape and r.shape == g[f"r{k}"].shape
        assert np.allclose(q, g[f"q{k}"], rtol=0, atol=1e-12)
        assert np.allclose(r, g[f"r{k}"], rtol=0, atol=1e-12)


# ------------------------------------------------------------------------- Krylov

def test_krylov_golden(ptg):
    g = load_golden("krylov.npz")
    h = g["h"]
    m = int(g["m"])
    alpha, beta, v = ptg.lanczos_iteration(lambda x: h @ x, g["v0"], m)
    assert rel(alpha, g["alpha"]) < 1e-12 and rel(beta, g["beta"]) < 1e-12
    assert rel(v, g["v"]) < 1e-10
    ex = ptg.expm_krylov(lambda x: h @ x, g["v0"], complex(g["dt"]), m, hermitian=True)
    assert rel(ex, g["expm"]) < 1e-12
    w, u = ptg.eigh_krylov(lambda x: h @ x, g["v0"], m, 2)
    assert rel(w, g["eig_w"]) < 1e-12
    for k in range(2):
        assert abs(abs(np.vdot(g["eig_u"][:, k], u[:, k])) - 1) < 1e-10
    d, U = ptg.eigh_tridiag(g["alpha"], g["beta"])
    dr, Ur = orc.eigh_tridiag(g["alpha"], g["beta"])
    assert np.allclose(d, dr, atol=1e-13)
    assert np.allclose(np.abs(np.sum(U * Ur, axis=0)), 1, atol=1e-10)


def test_krylov_breakdown(ptg):
    g = load_golden("krylov.npz")
    hs = g["hs"]
    with pytest.warns(RuntimeWarning):
        a2, b2, v2 = ptg.lanczos_iteration(lambda x: hs @ x, g["vs"], 8)
    assert a2.shape == g["alpha_bd"].shape and b2.shape == g["beta_bd"].shape
    assert rel(a2, g["alpha_bd"]) < 1e-12
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ex2 = ptg.expm_krylov(lambda x: hs @ x, g["vs"], -0.3j, 8, hermitian=True)
    assert rel(ex2, g["expm_bd"]) < 1e-12


# ------------------------------------------------------------------------ sweeps

def test_orthonormalize_matches_oracle(ptg):
    g = load_golden("tdvp_readme.npz")
    raw = golden_mps(g, "raw_")
    for mode in ("left", "right"):
        o = copy.deepcopy(raw)
        nrm_ref = orc.orthonormalize(o, mode)
        psi = as_ptg_mps(ptg, raw)
        nrm = psi.orthonormalize(mode)
        assert abs(nrm - nrm_ref) < 1e-12 * nrm_ref
        for x, y in zip(psi.a, o.a):
            assert x.shape == y.shape
            assert np.allclose(x, y, atol=1e-12)
        for qa, qb in zip(psi.qbonds, o.qbonds):
            assert np.array_equal(qa, qb)


def _run_tdvp_golden(ptg, name, graph=False, atol=1e-10):
    g = load_golden(name)
    h = golden_mpo(g, "h_")
    psi = as_ptg_mps(ptg, golden_mps(g, "p0_"))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = ptg.tdvp_singlesite(h, psi, complex(g["dt"]), int(g["numsteps"]),
                                  numiter_lanczos=int(g["m"]), graph=graph)
    ref = golden_mps(g, "p1_")
    assert abs(nrm - float(g["nrm"])) < 1e-12
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)                             # exact integers
    for x, y in zip(psi.a, ref.a):
        assert x.shape == y.shape
    # gauge-invariant: overlap with the reference state
    ov = orc.mps_vdot(ref, psi)
    assert abs(ov - orc.mps_vdot(ref, ref)) < atol * abs(orc.mps_vdot(ref, ref))
    return g, psi, h


def test_tdvp_readme_config(ptg):
    g, psi, h = _run_tdvp_golden(ptg, "tdvp_readme.npz")
    v = psi.to_vector()
    assert np.allclose(v, g["v1"], atol=1e-9)
    err = np.linalg.norm(v - g["exact"])
    err_ref = np.linalg.norm(g["v1"] - g["exact"])
    assert abs(err - err_ref) < 1e-9


def test_tdvp_quantum_numbers(ptg):
    g, psi, h = _run_tdvp_golden(ptg, "tdvp_qnum.npz")
    assert np.allclose(psi.to_vector(), g["v1"], atol=1e-10)
    assert np.allclose(psi.to_vector(), g["exact"], atol=2e-5)


def test_tdvp_xxz_bulk(ptg):
    g, psi, h = _run_tdvp_golden(ptg, "tdvp_xxz_bulk.npz")
    e1 = orc.mpo_average(psi, h)
    assert abs(e1 - complex(g["e1"])) < 1e-10 * max(1, abs(complex(g["e1"])))
    assert abs(ptg.mpo_average(psi, h) - e1) < 1e-11


def test_tdvp_ising_imaginary_time(ptg):
    g, psi, h = _run_tdvp_golden(ptg, "ising_imag.npz")
    assert np.allclose(psi.to_vector(), g["v1"], atol=1e-10)


def test_tdvp_graph_replay_equals_eager(ptg):
    g = load_golden("tdvp_xxz_bulk.npz")
    h = golden_mpo(g, "h_")
    p0 = golden_mps(g, "p0_")
    a = as_ptg_mps(ptg, p0)
    b = as_ptg_mps(ptg, p0)
    ptg.tdvp_singlesite(h, a, 0.05j, 4, numiter_lanczos=6, graph=False)
    ptg.tdvp_singlesite(h, b, 0.05j, 4, numiter_lanczos=6, graph=True)
    for x, y in zip(a.a, b.a):
        assert np.array_equal(x, y)


def test_tdvp_symmetry_reversibility(ptg):
    """test/test_tdvp.py:78-119: forward then backward returns to psi0 (1e-10)."""
    rng = np.random.default_rng(42)
    nsites = 10
    h = ptg.heisenberg_xxz_1d_mpo(nsites, 4.0 / 3, 5.0 / 13, -2.0 / 7)
    h.zero_qnumbers()
    qb = [np.array([0])] + [np.zeros(5, dtype=int) for _ in range(nsites - 1)] + [np.array([0])]
    psi = ptg.MPS(h.qsite, qb, fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    v0 = psi.to_vector()
    ptg.tdvp_singlesite(h, psi, 0.5j, 1, numiter_lanczos=10)
    ptg.tdvp_singlesite(h, psi, -0.5j, 1, numiter_lanczos=10)
    assert np.allclose(psi.to_vector(), v0, atol=1e-10)


def test_tdvp_larger_chain_vs_oracle(ptg):
    """L=24, D=32 real time, 2 steps: energy, norm and overlap vs the oracle (1e-10)."""
    rng = np.random.default_rng(7)
    L, D = 24, 32
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    o = orc.OMPS(psi.qsite, psi.qbonds, [x.copy() for x in psi.a])
    orc.tdvp_singlesite(h, o, 0.05j, 2, numiter_lanczos=8)
    ptg.tdvp_singlesite(h, psi, 0.05j, 2, numiter_lanczos=8)
    e_ref = orc.mpo_average(o, h)
    e = orc.mpo_average(psi, h)
    assert abs(e - e_ref) < 1e-10 * abs(e_ref)
    ov = orc.mps_vdot(o, psi)
    assert abs(abs(ov) - 1) < 1e-10 and abs(ov - 1) < 1e-9


def test_dmrg_singlesite_golden(ptg):
    g = load_golden("dmrg.npz")
    h = golden_mpo(g, "h_")
    psi = as_ptg_mps(ptg, golden_mps(g, "p0_"))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        en = ptg.dmrg_singlesite(h, psi, int(g["numsweeps"]))
    assert np.allclose(en, g["en"], rtol=0, atol=1e-11)
    assert abs(en[-1] - float(g["en_exact"])) < 1e-11
    ref = golden_mps(g, "p1_")
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    v = psi.to_vector()
    assert abs(abs(np.vdot(v, g["v1"])) - 1) < 1e-9


def test_run_measurements_on_device(ptg):
    """TDVPRun.energy / vdot contract the resident tensors on the device and agree
    with the oracle on the downloaded state (pytenet/chain_ops.py:151-189)."""
    rng = np.random.default_rng(8)
    L = 10
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), 8) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    run = ptg.TDVPRun(h, psi, numiter_lanczos=6)
    run.step(0.1j)
    e_dev, n_dev = run.energy(), run.norm()
    run.download()
    assert abs(e_dev - orc.mpo_average(psi, h)) < 1e-12 * max(1.0, abs(e_dev))
    assert abs(n_dev ** 2 - orc.mps_vdot(psi, psi).real) < 1e-12


def test_apply_mpo_golden(ptg):
    """apply_mpo on the GPU (pytenet/chain_ops.py:215-234) against the reference's
    output: integer bond quantum numbers bit-exact, tensors to 1e-13."""
    g = load_golden("apply_mpo.npz")
    h, p0, p1 = golden_mpo(g, "h_"), golden_mps(g, "p0_"), golden_mps(g, "p1_")
    out = ptg.apply_mpo(h, as_ptg_mps(ptg, p0))
    for qa, qb in zip(out.qbonds, p1.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(out.a, p1.a):
        assert x.shape == y.shape
        assert np.max(np.abs(x - y)) < 1e-13 * max(1.0, np.max(np.abs(y)))
