"""Two-site TDVP / DMRG on the GPU and the device SVD under them.

The reference splits with LAPACK's SVD, whose singular vectors carry a phase per
singular value that another SVD need not reproduce; the oracle test pins tensors
elementwise because the oracle calls LAPACK too. Here the comparison is on what
does not depend on that phase: bond dimensions and quantum numbers (bit-exact),
singular values, the state vector on the full Hilbert space, norms and energies
(pytenet/tdvp.py:121-220, pytenet/dmrg.py:96-178, pytenet/block_sparse_util.py:244-330)."""

import warnings

import numpy as np
import pytest

from conftest import golden_mpo, golden_mps, load_golden
from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ptg():
    import pytenet_gb300 as m
    from pytenet_gb300 import _lib
    _lib.load()
    return m


def dev_svd(a):
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import empty, ptr, stream_ptr, to_dev, to_host
    L = _lib.load()
    m, n = a.shape
    k = min(m, n)
    da, du, dv = to_dev(a), empty((m, k)), empty((k, n))
    ds = torch.zeros(k, dtype=torch.float64, device="cuda")
    sw = torch.zeros(1, dtype=torch.int32, device="cuda")
    wsb = L.ptn_svd_workspace_bytes(m, n)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(L.ptn_svd(ptr(da), m, n, n, ptr(du), k, ptr(ds), ptr(dv), n, ptr(sw), ptr(ws), wsb,
                         stream_ptr()))
    return to_host(du), ds.cpu().numpy(), to_host(dv), int(sw.item())


@pytest.mark.parametrize("mn", [(1, 1), (1, 5), (5, 1), (7, 3), (3, 7), (40, 64), (64, 40),
                                (128, 128), (200, 33)])
def test_svd_matches_lapack_values(ptg, mn):
    m, n = mn
    rng = np.random.default_rng(m * 100 + n)
    a = orc.crandn((m, n), rng)
    u, s, vh, sweeps = dev_svd(a)
    s_ref = np.linalg.svd(a, compute_uv=False)
    k = min(m, n)
    print("svd", mn, "sweeps", sweeps, "s err", np.abs(s - s_ref).max() / s_ref.max())
    assert sweeps < 60
    assert np.all(np.diff(s) <= 0)
    assert np.abs(s - s_ref).max() <= 1e-13 * s_ref.max()
    assert np.abs(u @ np.diag(s) @ vh - a).max() <= 1e-13 * s_ref.max() * np.sqrt(max(m, n))
    assert np.abs(u.conj().T @ u - np.eye(k)).max() < 1e-13
    assert np.abs(vh @ vh.conj().T - np.eye(k)).max() < 1e-13


def test_svd_rank_deficient_and_zero(ptg):
    rng = np.random.default_rng(2)
    a = orc.crandn((30, 6), rng) @ orc.crandn((6, 20), rng)
    u, s, vh, _ = dev_svd(a)
    s_ref = np.linalg.svd(a, compute_uv=False)
    assert np.abs(s - s_ref).max() <= 1e-13 * s_ref.max()
    assert np.abs(u @ np.diag(s) @ vh - a).max() <= 1e-12 * s_ref.max()
    # the six non-zero singular directions are orthonormal
    assert np.abs(u[:, :6].conj().T @ u[:, :6] - np.eye(6)).max() < 1e-13
    z = np.zeros((4, 3), dtype=complex)
    u, s, vh, _ = dev_svd(z)
    assert np.all(s == 0) and np.all(u @ np.diag(s) @ vh == 0)


def test_block_sparse_svd_matches_reference_structure(ptg):
    """Blocks, block order, quantum numbers and singular values as the oracle's
    LAPACK-based block_sparse_svd; the product u diag(s) v reproduces a."""
    rng = np.random.default_rng(3)
    for m, n in ((23, 15), (40, 12), (9, 20)):
        a = orc.crandn((m, n), rng)
        q0 = rng.integers(-2, 3, size=m)
        q1 = rng.integers(-2, 3, size=n)
        orc.enforce_qsparsity(a, [q0, -q1])
        u, s, v, q = ptg.block_sparse_svd(a, q0, q1)
        ur, sr, vr, qr = orc.block_sparse_svd(a, q0, q1)
        assert np.array_equal(q, qr)
        assert np.abs(s - sr).max() <= 1e-13 * max(1.0, sr.max())
        assert np.abs((u * s) @ v - a).max() <= 1e-13 * max(1.0, sr.max())
        assert orc.is_qsparse(u, [q0, -q]) and orc.is_qsparse(v, [q, -q1])
    # no common quantum number: the reference's placeholder factors
    a = np.zeros((4, 3), dtype=complex)
    u, s, v, q = ptg.block_sparse_svd(a, np.array([1, 1, 3, 5]), np.array([2, 4, 4]))
    assert u.shape == (4, 1) and u[0, 0] == 1 and np.all(s == 0) and np.array_equal(q, [1])


def psi_vector(p):
    return orc.mps_to_vector(p)


def test_twosite_tdvp_and_dmrg_match_reference(ptg):
    """The reference fixture (XXZ L=8 with quantum numbers, bonds grown from at most
    4 by the truncated splits): bond quantum numbers bit-exact after both sweeps,
    state vectors to 1e-10, returned norm, energy and DMRG energies to 1e-10."""
    g = load_golden("twosite.npz")
    h = golden_mpo(g, "h_")
    p0 = golden_mps(g, "p0_")
    psi = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
    psi.a = [x.copy() for x in p0.a]
    psi_d = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
    psi_d.a = [x.copy() for x in p0.a]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = ptg.tdvp_twosite(h, psi, complex(g["dt"]), int(g["numsteps"]),
                               numiter_lanczos=int(g["m"]), tol_split=float(g["tol"]))
        en = ptg.dmrg_twosite(h, psi_d, 2, numiter_lanczos=10, tol_split=1e-10)
    assert abs(nrm - float(g["nrm"])) < 1e-12 * max(1.0, abs(float(g["nrm"])))
    ref = golden_mps(g, "p1_")
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(psi.a, ref.a):
        assert x.shape == y.shape
    v = psi_vector(psi)
    dv = np.abs(v - g["v1"]).max() / np.abs(g["v1"]).max()
    e1 = orc.mpo_average(psi, h)
    print("two-site TDVP: state", dv, "energy", abs(e1 - complex(g["e1"])), "dmrg", en, g["en"])
    assert dv < 1e-10
    assert abs(e1 - complex(g["e1"])) < 1e-10 * max(1.0, abs(complex(g["e1"])))
    refd = golden_mps(g, "d1_")
    for qa, qb in zip(psi_d.qbonds, refd.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(psi_d.a, refd.a):
        assert x.shape == y.shape
    assert np.allclose(en, g["en"], rtol=0, atol=1e-10)
    # the DMRG state itself, up to a global phase
    vd, vr = psi_vector(psi_d), orc.mps_to_vector(refd)
    ph = np.vdot(vd, vr)
    assert abs(abs(ph) - 1) < 1e-10 and np.abs(vd * ph - vr).max() < 1e-8


def test_twosite_tdvp_tracks_oracle_larger(ptg):
    """A larger run than the fixture: XXZ L=10 with quantum numbers, bonds grown up
    to 32 by truncation at 1e-10, 3 real-time steps: same bonds and quantum numbers
    as the oracle (LAPACK splits), state vector to 1e-9."""
    rng = np.random.default_rng(17)
    L = 10
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    qb = [np.array([0])]
    for _ in range(L - 1):
        qb.append(np.sort(np.array([q + h.qsite for q in qb[-1]]).reshape(-1)))
    qb.append(np.array([2]))
    qb = [q if len(q) <= 6 else q[np.linspace(0, len(q) - 1, 6).astype(int)] for q in qb]
    psi = ptg.MPS(h.qsite, qb, fill="random", rng=rng)
    ref = orc.OMPS(psi.qsite, psi.qbonds, [x.copy() for x in psi.a])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        orc.tdvp_twosite(h, ref, 0.05j, 3, numiter_lanczos=8, tol_split=1e-10)
        ptg.tdvp_twosite(h, psi, 0.05j, 3, numiter_lanczos=8, tol_split=1e-10)
    for qa, qr_ in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qr_)
    v, vr = psi_vector(psi), orc.mps_to_vector(ref)
    print("two-site L=10 bonds", [len(q) for q in psi.qbonds], "state",
          np.abs(v - vr).max() / np.abs(vr).max())
    assert max(len(q) for q in psi.qbonds) > 6
    assert np.abs(v - vr).max() < 1e-9 * np.abs(vr).max()


def test_pair_components_match_oracle(ptg):
    """The pieces of one two-site step against the oracle: H_eff with the merged MPO
    pair (d*d = 4), one merged-pair Krylov exponential, one truncated split."""
    from pytenet_gb300.twosite import merge_mpo_pair
    rng = np.random.default_rng(23)
    h = ptg.heisenberg_xxz_1d_mpo(6, 1.0, 0.8, -0.1)
    Dl, Dm, Dr = 3, 5, 4
    a0 = orc.crandn((Dl, 2, Dm), rng)
    a1 = orc.crandn((Dm, 2, Dr), rng)
    x = orc._merge_pair(a0, a1)
    w2 = merge_mpo_pair(h.a[2], h.a[3])
    cl, cr = w2.shape[0], w2.shape[3]
    l = orc.crandn((Dl, cl, Dl), rng)
    r = orc.crandn((Dr, cr, Dr), rng)
    l = 0.5 * (l + l.conj().transpose(2, 1, 0))
    r = 0.5 * (r + r.conj().transpose(2, 1, 0))
    y = ptg.apply_local_hamiltonian(x, w2, l, r)
    yr = orc.apply_local_hamiltonian(x, w2, l, r)
    print("heff d=4", np.abs(y - yr).max() / np.abs(yr).max())
    assert np.abs(y - yr).max() < 1e-12 * np.abs(yr).max()
    # merged-pair expm through the two-site run's own call
    from pytenet_gb300.twosite import TwoSiteRun
    from pytenet_gb300.device import to_dev, to_host
    psi = ptg.MPS(h.qsite, [[0], [0] * 2, [0] * 3, [0] * Dl, [0] * Dr, [0] * 2, [0]], fill="random",
                  rng=rng)
    h.zero_qnumbers()
    run = TwoSiteRun(h, psi, 6)
    xd = to_dev(x)
    run.local_expm(xd, to_dev(w2), to_dev(l), to_dev(r), cl, cr, 0.05j)
    xr = orc._site_step(l, r, w2, x, 0.05j, 6)
    print("pair expm", np.abs(to_host(xd) - xr).max() / np.abs(xr).max())
    assert np.abs(to_host(xd) - xr).max() < 1e-11 * np.abs(xr).max()


def test_compress_svd_matches_reference(ptg):
    """MPS.compress(tol, "svd", left / right) on the device (pytenet/mps.py:180-236)
    against the reference fixture: truncated bond dimensions and quantum numbers
    bit-exact, norm and compression factor to 1e-12, the compressed state to 1e-10."""
    g = load_golden("compress.npz")
    p0 = golden_mps(g, "p0_")
    for direction in ("left", "right"):
        psi = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
        psi.a = [x.copy() for x in p0.a]
        nrm, scale = psi.compress(1e-6, mode="svd", direction=direction)
        ref = golden_mps(g, f"{direction}_")
        assert abs(nrm - float(g[f"{direction}_nrm"])) < 1e-12 * abs(float(g[f"{direction}_nrm"]))
        assert abs(scale - float(g[f"{direction}_scale"])) < 1e-12
        for qa, qb in zip(psi.qbonds, ref.qbonds):
            assert np.array_equal(qa, qb)
        for x, y in zip(psi.a, ref.a):
            assert x.shape == y.shape
        v, vr = psi_vector(psi), orc.mps_to_vector(ref)
        print("compress", direction, "bonds", [len(q) for q in psi.qbonds], "state",
              np.abs(v - vr).max())
        assert np.abs(v - vr).max() < 1e-10 * max(1.0, np.abs(vr).max())


def test_compress_density_matches_reference(ptg):
    """MPS.compress(tol, "density") on the device (pytenet/mps.py:238-290): density
    matrices from FP64 GEMMs, eigenvectors per quantum-number block from the device
    SVD in the reference's block and eigenvalue order. Against the reference
    fixture: bond dimensions and quantum numbers bit-exact, norm and compression
    factor to 1e-12, the compressed state to 1e-10; the svd and density results
    describe states of the same norm."""
    g = load_golden("compress.npz")
    p0 = golden_mps(g, "p0_")
    psi = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
    psi.a = [x.copy() for x in p0.a]
    nrm, scale = psi.compress(1e-6, mode="density")
    ref = golden_mps(g, "density_")
    assert abs(nrm - float(g["density_nrm"])) < 1e-12 * abs(float(g["density_nrm"]))
    assert abs(scale - float(g["density_scale"])) < 1e-12
    for qa, qb in zip(psi.qbonds, ref.qbonds):
        assert np.array_equal(qa, qb)
    for x, y in zip(psi.a, ref.a):
        assert x.shape == y.shape
    v = psi_vector(psi)
    vr = g["density_v"]
    print("compress density bonds", [len(q) for q in psi.qbonds], "state", np.abs(v - vr).max())
    assert np.abs(v - vr).max() < 1e-10 * max(1.0, np.abs(vr).max())
    assert abs(np.linalg.norm(v) - 1.0) < 1e-12
