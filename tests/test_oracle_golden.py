"""Pin the CPU oracle against golden outputs of the reference itself
(fixtures made by tests/golden/gen_golden.py). CPU only."""

import copy
import warnings

import numpy as np
import pytest

from conftest import load_golden, golden_mps, golden_mpo
from oracle import ptn_oracle as orc

RTOL = 1e-12


def rel(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)


def test_chain_ops_match_reference():
    g = load_golden("chain_ops.npz")
    assert rel(orc.apply_local_hamiltonian(g["a"], g["w"], g["l"], g["r"]), g["heff"]) < RTOL
    assert rel(orc.apply_local_hamiltonian(g["a"], g["wc"], g["l"], g["r"]), g["heff_c"]) < RTOL
    assert rel(orc.apply_local_bond_contraction(g["c"], g["lb"], g["r"]), g["bond"]) < RTOL
    assert rel(orc.env_step_left(g["a"], g["b"], g["w"], g["l"]), g["env_left"]) < RTOL
    assert rel(orc.env_step_right(g["a"], g["b"], g["w"], g["r"]), g["env_right"]) < RTOL
    assert rel(orc.env_step_left(g["a"], g["a"], g["wc"], g["l"]), g["env_left_aa"]) < RTOL
    assert rel(orc.env_step_right(g["a"], g["a"], g["wc"], g["r"]), g["env_right_aa"]) < RTOL


def test_krylov_match_reference():
    g = load_golden("krylov.npz")
    h = g["h"]
    m = int(g["m"])
    alpha, beta, v = orc.lanczos_iteration(lambda x: h @ x, g["v0"], m)
    assert rel(alpha, g["alpha"]) < RTOL and rel(beta, g["beta"]) < RTOL
    assert rel(v, g["v"]) < 1e-10
    ex = orc.expm_krylov(lambda x: h @ x, g["v0"], complex(g["dt"]), m)
    assert rel(ex, g["expm"]) < RTOL
    w, u = orc.eigh_krylov(lambda x: h @ x, g["v0"], m, 2)
    assert rel(w, g["eig_w"]) < RTOL
    # Ritz vectors are defined up to sign
    for k in range(2):
        s = np.vdot(g["eig_u"][:, k], u[:, k])
        assert abs(abs(s) - 1) < 1e-10


def test_krylov_breakdown_truncates_like_reference():
    g = load_golden("krylov.npz")
    hs = g["hs"]
    with pytest.warns(RuntimeWarning):
        a2, b2, v2 = orc.lanczos_iteration(lambda x: hs @ x, g["vs"], 8)
    assert a2.shape == g["alpha_bd"].shape and b2.shape == g["beta_bd"].shape
    assert rel(a2, g["alpha_bd"]) < RTOL
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ex2 = orc.expm_krylov(lambda x: hs @ x, g["vs"], -0.3j, 8)
    assert rel(ex2, g["expm_bd"]) < RTOL


def test_block_sparse_qr_match_reference():
    g = load_golden("block_qr.npz")
    for k in range(int(g["ncases"])):
        a, q0, q1 = g[f"a{k}"], g[f"q0_{k}"], g[f"q1_{k}"]
        q, r, qi = orc.block_sparse_qr(a, q0, q1)
        # integer bookkeeping is bit-exact
        assert np.array_equal(qi, g[f"qi{k}"])
        assert q.shape == g[f"q{k}"].shape and r.shape == g[f"r{k}"].shape
        assert np.allclose(q, g[f"q{k}"], rtol=0, atol=1e-12)
        assert np.allclose(r, g[f"r{k}"], rtol=0, atol=1e-12)
        assert np.allclose(q @ r, a, atol=1e-12)


def test_mpo_to_matrix_matches_reference():
    g = load_golden("mpos.npz")
    for L in (2, 3, 4, 5, 6):
        for name in ("xxz", "ising"):
            op = golden_mpo(g, f"{name}{L}_")
            assert np.allclose(orc.mpo_to_matrix(op), g[f"{name}{L}_mat"], rtol=0, atol=1e-14)


def test_mps_random_draw_order():
    g = load_golden("mps_random.npz")
    ref = golden_mps(g, "r_")
    psi = orc.random_mps(ref.qsite, ref.qbonds, np.random.default_rng(1009))
    for x, y in zip(psi.a, ref.a):
        assert np.array_equal(x, y)


def _check_tdvp(name, atol_vec=1e-10):
    g = load_golden(name)
    h = golden_mpo(g, "h_")
    psi = golden_mps(g, "p0_")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = orc.tdvp_singlesite(h, psi, complex(g["dt"]), int(g["numsteps"]), int(g["m"]))
    ref = golden_mps(g, "p1_")
    assert abs(nrm - float(g["nrm"])) < 1e-12
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(psi.a, ref.a):
        assert x.shape == y.shape
        assert np.allclose(x, y, rtol=0, atol=atol_vec)
    return g, psi


def test_tdvp_readme_config():
    g, psi = _check_tdvp("tdvp_readme.npz")
    v = orc.mps_to_vector(psi)
    assert np.allclose(v, g["v1"], atol=1e-10)
    # fixed-bond projection error equals the reference's own error vs exact
    err = np.linalg.norm(v - g["exact"])
    err_ref = np.linalg.norm(g["v1"] - g["exact"])
    assert abs(err - err_ref) < 1e-10


def test_tdvp_quantum_numbers():
    g, psi = _check_tdvp("tdvp_qnum.npz")
    assert np.allclose(orc.mps_to_vector(psi), g["exact"], atol=2e-5)


def test_tdvp_xxz_bulk():
    g, psi = _check_tdvp("tdvp_xxz_bulk.npz")
    h = golden_mpo(g, "h_")
    assert abs(orc.mpo_average(psi, h) - complex(g["e1"])) < 1e-10


def test_tdvp_ising_imaginary_time():
    g, psi = _check_tdvp("ising_imag.npz")
    assert np.allclose(orc.mps_to_vector(psi), g["v1"], atol=1e-10)


def test_dmrg_singlesite():
    g = load_golden("dmrg.npz")
    h = golden_mpo(g, "h_")
    psi = golden_mps(g, "p0_")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        en = orc.dmrg_singlesite(h, psi, int(g["numsweeps"]))
    assert np.allclose(en, g["en"], rtol=0, atol=1e-12)
    assert abs(en[-1] - float(g["en_exact"])) < 1e-12
    ref = golden_mps(g, "p1_")
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    v = orc.mps_to_vector(psi)
    # eigenvector up to a global phase
    assert abs(abs(np.vdot(v, g["v1"])) - 1) < 1e-10


def test_mlp_oracle_gradient_by_finite_differences():
    """Pin the NumPy MLP checker itself: analytic gradient vs central differences."""
    from oracle import mlp_oracle
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, 5057)
    X = rng.normal(size=(7, 12))
    T = rng.uniform(size=7)
    g, loss = mlp_oracle.mlp_grad(p, X, T)
    for idx in [0, 5, 770, 900, 4900, 4950, 5000, 5056]:
        e = np.zeros_like(p)
        e[idx] = 1e-6
        fd = (np.mean((mlp_oracle.mlp_forward(p + e, X) - T) ** 2) -
              np.mean((mlp_oracle.mlp_forward(p - e, X) - T) ** 2)) / 2e-6
        assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(g[idx]))


def test_apply_mpo_matches_reference():
    """chain_ops.py:215-234 with quantum numbers: tensors and flattened bond qnumbers."""
    g = load_golden("apply_mpo.npz")
    h, p0, p1 = golden_mpo(g, "h_"), golden_mps(g, "p0_"), golden_mps(g, "p1_")
    out = orc.apply_mpo(h, p0)
    for qa, qb in zip(out.qbonds, p1.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(out.a, p1.a):
        assert x.shape == y.shape and np.allclose(x, y, rtol=0, atol=1e-14)


def test_twosite_tdvp_and_dmrg_match_reference():
    """Two-site TDVP (tdvp.py:121-220) and DMRG (dmrg.py:96-178) with quantum numbers
    and truncated block-sparse SVD: bond dimensions and quantum numbers bit-exact,
    tensors, norm and energies to 1e-10."""
    g = load_golden("twosite.npz")
    h = golden_mpo(g, "h_")
    psi = golden_mps(g, "p0_")
    psi_d = golden_mps(g, "p0_")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = orc.tdvp_twosite(h, psi, complex(g["dt"]), int(g["numsteps"]), int(g["m"]),
                               float(g["tol"]))
        en = orc.dmrg_twosite(h, psi_d, 2, 10, 1e-10)
    assert abs(nrm - float(g["nrm"])) < 1e-12 * max(1.0, abs(float(g["nrm"])))
    for name, out in (("p1_", psi), ("d1_", psi_d)):
        ref = golden_mps(g, name)
        for qa, qb in zip(out.qbonds, ref.qbonds):
            assert np.array_equal(qa, qb)
        for x, y in zip(out.a, ref.a):
            assert x.shape == y.shape
            assert np.allclose(x, y, rtol=0, atol=1e-10 * max(1.0, np.max(np.abs(y))))
    assert np.allclose(en, g["en"], rtol=0, atol=1e-12)
    assert np.allclose(orc.mps_to_vector(psi), g["v1"], atol=1e-10 * np.max(np.abs(g["v1"])))
    assert abs(orc.mpo_average(psi, h) - complex(g["e1"])) < 1e-10 * max(1.0, abs(complex(g["e1"])))


def test_truncation_rule_matches_reference_semantics():
    """retained_bond_indices (bond_ops.py:23-38): keep the values whose normalised
    squares, accumulated from the smallest, exceed tol; zero vector keeps nothing."""
    s = np.array([1.0, 1e-3, 0.5, 1e-6, 0.0])
    assert list(orc.retained_bond_indices(s.copy(), 0)) == [0, 1, 2, 3]
    # (1e-3)^2 / 1.25 accumulated with the smaller ones stays below 1e-5: dropped
    assert list(orc.retained_bond_indices(s.copy(), 1e-5)) == [0, 2]
    assert list(orc.retained_bond_indices(np.zeros(3), 0.1)) == []


def test_compress_svd_matches_reference():
    """MPS.compress(tol, "svd", left / right) (mps.py:180-236): truncated bond
    dimensions and quantum numbers bit-exact, tensors, norm and scale to 1e-10."""
    g = load_golden("compress.npz")
    for direction in ("left", "right"):
        psi = golden_mps(g, "p0_")
        nrm, scale = orc.compress_svd(psi, 1e-6, direction)
        ref = golden_mps(g, f"{direction}_")
        assert abs(nrm - float(g[f"{direction}_nrm"])) < 1e-12 * abs(float(g[f"{direction}_nrm"]))
        assert abs(scale - float(g[f"{direction}_scale"])) < 1e-12
        for qa, qb in zip(psi.qbonds, ref.qbonds):
            assert np.array_equal(qa, qb)
        for x, y in zip(psi.a, ref.a):
            assert x.shape == y.shape
            assert np.allclose(x, y, rtol=0, atol=1e-10)


def test_compress_density_matches_reference():
    """MPS.compress(tol, "density") (mps.py:238-290, block_sparse_eigh of
    block_sparse_util.py:183-241): bond dimensions and quantum numbers bit-exact
    (blocks in the order of the Python set of the row quantum numbers), tensors,
    norm and scale to 1e-12."""
    g = load_golden("compress.npz")
    psi = golden_mps(g, "p0_")
    nrm, scale = orc.compress_density(psi, 1e-6)
    ref = golden_mps(g, "density_")
    assert abs(nrm - float(g["density_nrm"])) < 1e-12 * abs(float(g["density_nrm"]))
    assert abs(scale - float(g["density_scale"])) < 1e-12
    assert [len(q) for q in psi.qbonds] != [len(q) for q in golden_mps(g, "p0_").qbonds]
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(psi.a, ref.a):
        assert x.shape == y.shape
        assert np.allclose(x, y, rtol=0, atol=1e-12)
    assert np.allclose(orc.mps_to_vector(psi), g["density_v"], rtol=0, atol=1e-12)


def test_xxz_l64_fixture_input_and_initial_state():
    """The L=64, D=256 fixture (whole trajectory checked on the GPU): its input is
    regenerated from the seed with the reference's draw order, bit for bit, and
    the left-orthonormalised initial state gives the reference's step-0
    fingerprints (energy, norm, weighted one-site observables)."""
    g = load_golden("tdvp_xxz_l64.npz")
    h, mz, mx = golden_mpo(g, "h_"), golden_mpo(g, "mz_"), golden_mpo(g, "mx_")
    rng = np.random.default_rng(int(g["seed"]))
    psi = orc.random_mps(h.qsite, [np.zeros(bi, dtype=int) for bi in g["bonds"]], rng)
    assert np.array_equal(np.array([x.sum() for x in psi.a]), g["raw_sum"])
    assert np.array_equal(np.array([x.reshape(-1)[0] for x in psi.a]), g["raw_first"])
    orc.orthonormalize(psi, mode="left")
    e = orc.mpo_average(psi, h)
    assert abs(e - g["energy"][0]) < 1e-12 * abs(g["energy"][0])
    assert abs(orc.mps_norm(psi) - g["norm"][0]) < 1e-12
    assert abs(orc.mpo_average(psi, mz) - g["obs_z"][0]) < 1e-12 * max(abs(g["obs_z"][0]), 1e-3)
    assert abs(orc.mpo_average(psi, mx) - g["obs_x"][0]) < 1e-12 * max(abs(g["obs_x"][0]), 1e-3)
