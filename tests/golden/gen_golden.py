"""
Generate golden fixtures by running the PyTeNet reference itself with fixed seeds.

Run in a container where the reference checkout exists:

    PTN_REFERENCE=<reference checkout> python tests/golden/gen_golden.py [fixture ...]

The reference's own tests draw from unseeded generators, so it ships no golden
vectors; this script makes them. Every fixture stores the exact inputs that
were handed to the reference (MPO tensors, MPS tensors, quantum numbers) and
the reference's outputs, so the oracle and the GPU engine can be run on the
identical inputs without the reference present.
"""

import copy
import os
import sys
import numpy as np
from scipy.linalg import expm

# the reference checkout to run: PTN_REFERENCE, else an installed `pytenet`
if os.environ.get("PTN_REFERENCE"):
    sys.path.insert(0, os.environ["PTN_REFERENCE"])
import pytenet as ptn  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def pack_list(prefix, arrs):
    return {f"{prefix}{i}": np.asarray(x) for i, x in enumerate(arrs)}


def pack_mps(prefix, psi):
    d = {f"{prefix}qsite": np.asarray(psi.qsite), f"{prefix}n": np.array(psi.nsites)}
    d.update(pack_list(prefix + "a", psi.a))
    d.update(pack_list(prefix + "qb", psi.qbonds))
    return d


def pack_mpo(prefix, op):
    d = {f"{prefix}qsite": np.asarray(op.qsite), f"{prefix}n": np.array(op.nsites)}
    d.update(pack_list(prefix + "w", op.a))
    d.update(pack_list(prefix + "qb", op.qbonds))
    return d


def save(name, **kw):
    path = os.path.join(OUT, name)
    np.savez_compressed(path, **kw)
    print("wrote", path, os.path.getsize(path), "bytes")


def gen_chain_ops():
    rng = np.random.default_rng(1001)
    Dl, d, Dr, chl, chr_ = 5, 2, 7, 3, 4
    a = ptn.crandn((Dl, d, Dr), rng)
    b = ptn.crandn((Dl, d, Dr), rng)
    w = rng.normal(size=(chl, d, d, chr_))
    wc = ptn.crandn((chl, d, d, chr_), rng)
    l = ptn.crandn((Dl, chl, Dl), rng)
    r = ptn.crandn((Dr, chr_, Dr), rng)
    c = ptn.crandn((Dl, Dr), rng)
    lb = ptn.crandn((Dl, chr_, Dl), rng)
    save("chain_ops.npz", a=a, b=b, w=w, wc=wc, l=l, r=r, c=c, lb=lb,
         heff=ptn.apply_local_hamiltonian(a, w, l, r),
         heff_c=ptn.apply_local_hamiltonian(a, wc, l, r),
         bond=ptn.apply_local_bond_contraction(c, lb, r),
         env_left=ptn.contraction_operator_step_left(a, b, w, l),
         env_right=ptn.contraction_operator_step_right(a, b, w, r),
         env_left_aa=ptn.contraction_operator_step_left(a, a, wc, l),
         env_right_aa=ptn.contraction_operator_step_right(a, a, wc, r))


def gen_krylov():
    rng = np.random.default_rng(1002)
    n, m = 96, 12
    h = ptn.crandn((n, n), rng) / np.sqrt(n)
    h = 0.5 * (h + h.conj().T)
    v0 = ptn.crandn(n, rng) / np.sqrt(n)
    alpha, beta, v = ptn.lanczos_iteration(lambda x: h @ x, v0, m)
    dt = 0.4 + 0.2j
    ex = ptn.expm_krylov(lambda x: h @ x, v0, dt, m, hermitian=True)
    ew, eu = ptn.eigh_krylov(lambda x: h @ x, v0, m, 2)
    # breakdown: Krylov space exhausted after 4 vectors
    hs = np.diag([0.3, -1.2, 0.7, 2.0]).astype(complex)
    vs = np.array([1.0, 0.5 - 0.2j, -0.3j, 0.25])
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        a2, b2, v2 = ptn.lanczos_iteration(lambda x: hs @ x, vs, 8)
        ex2 = ptn.expm_krylov(lambda x: hs @ x, vs, -0.3j, 8, hermitian=True)
    save("krylov.npz", h=h, v0=v0, m=np.array(m), dt=np.array(dt), alpha=alpha, beta=beta, v=v,
         expm=ex, eig_w=ew, eig_u=eu, hs=hs, vs=vs, alpha_bd=a2, beta_bd=b2, v_bd=v2,
         expm_bd=ex2)


def gen_block_qr():
    rng = np.random.default_rng(1003)
    out = {}
    cases = [(23, 15, True), (40, 12, True), (9, 20, True), (30, 30, False), (64, 32, False)]
    for k, (m, n, qn) in enumerate(cases):
        a = ptn.crandn((m, n), rng)
        if qn:
            q0 = rng.integers(-2, 3, size=m)
            q1 = rng.integers(-2, 3, size=n)
        else:
            q0 = np.zeros(m, dtype=int)
            q1 = np.zeros(n, dtype=int)
        ptn.enforce_qsparsity(a, [q0, -q1])
        if k == 4:
            a[:, 20:] = 0   # rank-deficient: trailing zero columns
        q, r, qi = ptn.block_sparse_qr(a, q0, q1)
        out.update({f"a{k}": a, f"q0_{k}": q0, f"q1_{k}": q1, f"q{k}": q, f"r{k}": r,
                    f"qi{k}": qi})
    # no common quantum numbers
    a = np.zeros((4, 3), dtype=complex)
    q0 = np.array([1, 1, 3, 5])
    q1 = np.array([2, 4, 4])
    q, r, qi = ptn.block_sparse_qr(a, q0, q1)
    out.update({"a5": a, "q0_5": q0, "q1_5": q1, "q5": q, "r5": r, "qi5": qi})
    out["ncases"] = np.array(6)
    save("block_qr.npz", **out)


def gen_mpos():
    out = {}
    for L in (2, 3, 4, 5, 6):
        h = ptn.heisenberg_xxz_1d_mpo(L, 1.3, 0.7, -0.2)
        out.update(pack_mpo(f"xxz{L}_", h))
        out[f"xxz{L}_mat"] = h.to_matrix()
        g = ptn.ising_1d_mpo(L, 1.0, 0.15, 0.8)
        out.update(pack_mpo(f"ising{L}_", g))
        out[f"ising{L}_mat"] = g.to_matrix()
    save("mpos.npz", **out)


def gen_tdvp_readme():
    """Config of the reference README (README.rst:20-47), seeded."""
    rng = np.random.default_rng(1004)
    nsites = 10
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [1, 2, 4, 8, 16, 28, 16, 8, 4, 2, 1]
    psi = ptn.MPS(h.qsite, [bi*[0] for bi in b], fill="random", rng=rng)
    raw = copy.deepcopy(psi)
    for i in range(nsites):
        psi.a[i][8:, :, :] = 0
        psi.a[i][:, :, 8:] = 0
    psi.orthonormalize(mode="left")
    psi0 = copy.deepcopy(psi)
    dt, numsteps, m = 0.01 - 0.05j, 100, 5
    exact = expm(-dt*numsteps*h.to_matrix()) @ psi0.to_vector()
    nrm = ptn.tdvp_singlesite(h, psi, dt, numsteps, numiter_lanczos=m)
    save("tdvp_readme.npz", **pack_mpo("h_", h), **pack_mps("raw_", raw), **pack_mps("p0_", psi0),
         **pack_mps("p1_", psi), nrm=np.array(nrm), dt=np.array(dt), numsteps=np.array(numsteps),
         m=np.array(m), v1=psi.to_vector(), exact=exact,
         energy=np.array(ptn.mpo_average(psi, h)))


def gen_tdvp_qnum():
    """Quantum-number conserving setup of test/test_tdvp.py:7-75, seeded, fewer steps."""
    rng = np.random.default_rng(1005)
    nsites = 8
    dt, numsteps, m = 0.02 - 0.05j, 4, 5
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 4.0/3, 5.0/13, -2.0/7)
    spin_tot = 2
    qbonds = [np.array([0])]
    for _ in range(nsites - 1):
        qbonds.append(np.sort(np.array([q + h.qsite for q in qbonds[-1]]).reshape(-1)))
    qbonds.append(np.array([2*spin_tot]))
    psi = ptn.MPS(h.qsite, qbonds, fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    psi.orthonormalize(mode="right")
    for i in range(nsites):
        psi.a[i][8:, :, :] = 0
        psi.a[i][:, :, 8:] = 0
    psi.orthonormalize(mode="left")
    psi0 = copy.deepcopy(psi)
    exact = expm(-dt*numsteps*h.to_matrix()) @ psi0.to_vector()
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = ptn.tdvp_singlesite(h, psi, dt, numsteps, numiter_lanczos=m)
    save("tdvp_qnum.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi0), **pack_mps("p1_", psi),
         nrm=np.array(nrm), dt=np.array(dt), numsteps=np.array(numsteps), m=np.array(m),
         v1=psi.to_vector(), exact=exact)


def gen_dmrg():
    """Setup of test/test_dmrg.py:5-49, seeded."""
    rng = np.random.default_rng(1006)
    nsites, numsweeps = 8, 4
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 4/5, 8/3, -2/7)
    psi = ptn.MPS.construct_random(nsites, h.qsite, 0, max_vdim=32, dtype="real", rng=rng)
    psi0 = copy.deepcopy(psi)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        en = ptn.dmrg_singlesite(h, psi, numsweeps)
    en_ref = np.linalg.eigvalsh(h.to_matrix())[0]
    save("dmrg.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi0), **pack_mps("p1_", psi),
         en=en, en_exact=np.array(en_ref), numsweeps=np.array(numsweeps), v1=psi.to_vector())


def gen_tdvp_xxz_bulk():
    """Scaled-down version of the L=64 real-time workload: uniform bond cap,
    zero quantum numbers, seeded complex Gaussian entries, left-orthonormalised."""
    rng = np.random.default_rng(1007)
    nsites, D = 12, 12
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2**min(i, nsites - i), D) for i in range(nsites + 1)]
    psi = ptn.MPS(h.qsite, [bi*[0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    psi0 = copy.deepcopy(psi)
    dt, numsteps, m = 0.05j, 3, 10
    e0 = ptn.mpo_average(psi0, h)
    nrm = ptn.tdvp_singlesite(h, psi, dt, numsteps, numiter_lanczos=m)
    save("tdvp_xxz_bulk.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi0), **pack_mps("p1_", psi),
         nrm=np.array(nrm), dt=np.array(dt), numsteps=np.array(numsteps), m=np.array(m),
         e0=np.array(e0), e1=np.array(ptn.mpo_average(psi, h)),
         overlap=np.array(ptn.mps_vdot(psi0, psi)))


def gen_ising_imag():
    """Scaled-down instance of the batched Ising workload: imaginary time."""
    rng = np.random.default_rng(1008)
    nsites, D = 10, 8
    h = ptn.ising_1d_mpo(nsites, 1.0, 0.1, 0.9)
    b = [min(2**min(i, nsites - i), D) for i in range(nsites + 1)]
    psi = ptn.MPS(h.qsite, [bi*[0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    psi0 = copy.deepcopy(psi)
    dt, numsteps, m = 0.05, 5, 8
    nrm = ptn.tdvp_singlesite(h, psi, dt, numsteps, numiter_lanczos=m)
    save("ising_imag.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi0), **pack_mps("p1_", psi),
         nrm=np.array(nrm), dt=np.array(dt), numsteps=np.array(numsteps), m=np.array(m),
         e1=np.array(ptn.mpo_average(psi, h)), v1=psi.to_vector())


def gen_mps_random():
    """Draw order of MPS(..., fill="random") and MPS.construct_random."""
    rng = np.random.default_rng(1009)
    qsite = [1, -1]
    qbonds = [[0], [1, -1], [2, 0, 0, -2], [1, -1, 1], [0]]
    psi = ptn.MPS(qsite, qbonds, fill="random", rng=rng)
    rng2 = np.random.default_rng(1010)
    psi2 = ptn.MPS.construct_random(7, qsite, 1, max_vdim=6, dtype="complex", rng=rng2)
    rng3 = np.random.default_rng(1011)
    psi3 = ptn.MPS.construct_random(6, qsite, 0, max_vdim=5, dtype="real", rng=rng3)
    save("mps_random.npz", **pack_mps("r_", psi), **pack_mps("c_", psi2), **pack_mps("d_", psi3))


def gen_apply_mpo():
    """apply_mpo (chain_ops.py:215-234) with non-trivial quantum numbers: XXZ MPO on
    a random quantum-number-sparse MPS of total spin 2 (the setup of test_tdvp.py)."""
    rng = np.random.default_rng(1012)
    nsites = 6
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 1.0, 0.8, -0.1)
    qbonds = [np.array([0])]
    for _ in range(nsites - 1):
        qbonds.append(np.sort(np.array([q + h.qsite for q in qbonds[-1]]).reshape(-1)))
    qbonds.append(np.array([2]))
    psi = ptn.MPS(h.qsite, qbonds, fill="random", rng=rng)
    op_psi = ptn.apply_mpo(h, psi)
    save("apply_mpo.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi), **pack_mps("p1_", op_psi))


def gen_twosite():
    """Two-site TDVP (tdvp.py:121-220) and DMRG (dmrg.py:96-178) with quantum numbers
    and SVD truncation: the bond dimensions grow from a small start."""
    rng = np.random.default_rng(1013)
    nsites = 8
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 1.0, 0.8, -0.1)
    qbonds = [np.array([0])]
    for _ in range(nsites - 1):
        qbonds.append(np.sort(np.array([q + h.qsite for q in qbonds[-1]]).reshape(-1)))
    qbonds.append(np.array([2]))
    # clamp the bonds to at most 4 entries (same sector structure) so that the
    # two-site steps have room to grow them
    qbonds = [q if len(q) <= 4 else q[np.linspace(0, len(q) - 1, 4).astype(int)] for q in qbonds]
    psi = ptn.MPS(h.qsite, qbonds, fill="random", rng=rng)
    psi0 = copy.deepcopy(psi)
    dt, numsteps, m, tol = 0.05 - 0.02j, 2, 6, 1e-8
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nrm = ptn.tdvp_twosite(h, psi, dt, numsteps, numiter_lanczos=m, tol_split=tol)
        psi_d = copy.deepcopy(psi0)
        en = ptn.dmrg_twosite(h, psi_d, 2, numiter_lanczos=10, tol_split=1e-10)
    save("twosite.npz", **pack_mpo("h_", h), **pack_mps("p0_", psi0), **pack_mps("p1_", psi),
         **pack_mps("d1_", psi_d), nrm=np.array(nrm), dt=np.array(dt),
         numsteps=np.array(numsteps), m=np.array(m), tol=np.array(tol), en=en,
         v1=psi.to_vector(), e1=np.array(ptn.mpo_average(psi, h)))


def gen_compress():
    """MPS.compress(tol, "svd", direction) (mps.py:180-236) and MPS.compress(tol,
    "density") (mps.py:238-290) on an MPS with quantum numbers whose bonds carry
    more than the state needs: an MPO applied to a state."""
    rng = np.random.default_rng(1014)
    nsites = 7
    h = ptn.heisenberg_xxz_1d_mpo(nsites, 1.0, 0.8, -0.1)
    qbonds = [np.array([0])]
    for _ in range(nsites - 1):
        qbonds.append(np.sort(np.array([q + h.qsite for q in qbonds[-1]]).reshape(-1)))
    qbonds.append(np.array([1]))
    psi = ptn.apply_mpo(h, ptn.MPS(h.qsite, qbonds, fill="random", rng=rng))
    out = {}
    out.update(pack_mps("p0_", psi))
    for direction in ("left", "right"):
        p = copy.deepcopy(psi)
        nrm, scale = p.compress(1e-6, mode="svd", direction=direction)
        out.update(pack_mps(f"{direction}_", p))
        out[f"{direction}_nrm"] = np.array(nrm)
        out[f"{direction}_scale"] = np.array(scale)
    p = copy.deepcopy(psi)
    nrm, scale = p.compress(1e-6, mode="density")
    out.update(pack_mps("density_", p))
    out["density_nrm"] = np.array(nrm)
    out["density_scale"] = np.array(scale)
    out["density_v"] = p.to_vector()
    save("compress.npz", **out)


def weighted_site_mpo(qsite, op, weights):
    """MPO of sum_i weights[i] op_i (bond 2: "not yet placed" / "placed"), zero
    quantum numbers, in the reference's layout (chil, d, d, chir)."""
    L, d = len(weights), op.shape[0]
    ident = np.identity(d)
    mpo = ptn.MPO(qsite, [[0]] + (L - 1) * [[0, 0]] + [[0]], fill="postpone")
    for i in range(L):
        w = np.zeros((2, d, d, 2))
        w[0, :, :, 0] = ident
        w[0, :, :, 1] = weights[i] * op
        w[1, :, :, 1] = ident
        if i == 0:
            w = w[:1]
        if i == L - 1:
            w = w[:, :, :, 1:]
        mpo.a[i] = w
    return mpo


def gen_tdvp_xxz_l64():
    """Plain complex128 at scale: XXZ L=64 (J=1, Delta=0.8, h=-0.1, zero quantum
    numbers), bonds min(2^min(i, L-i), 256), seeded complex Gaussian entries,
    left-orthonormalised; real time dt=0.05j, 20 steps of the reference's own
    tdvp_singlesite (one call per step), numiter_lanczos=10. The state (134 MB)
    is not stored: its draws are regenerated from the seed (the draw order is
    pinned by mps_random.npz) and checked against stored checksums; after every
    step the fixture keeps gauge-invariant fingerprints: energy, norm, the
    returned norm, two weighted one-site observables and the overlap with the
    initial state."""
    import time
    seed, L, D, dt, numsteps, m = 2064, 64, 256, 0.05j, 20, 10
    rng = np.random.default_rng(seed)
    h = ptn.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2**min(i, L - i), D) for i in range(L + 1)]
    psi = ptn.MPS(h.qsite, [bi*[0] for bi in b], fill="random", rng=rng)
    raw_sum = np.array([x.sum() for x in psi.a])
    raw_first = np.array([x.reshape(-1)[0] for x in psi.a])
    psi.orthonormalize(mode="left")
    psi0 = copy.deepcopy(psi)
    wrng = np.random.default_rng(seed + 1)
    cz, cx = wrng.uniform(-1, 1, L), wrng.uniform(-1, 1, L)
    sz = np.array([[0.5, 0.0], [0.0, -0.5]])
    sx = np.array([[0.0, 0.5], [0.5, 0.0]])
    mz = weighted_site_mpo(h.qsite, sz, cz)
    mx = weighted_site_mpo(h.qsite, sx, cx)

    def fingerprint(p):
        return [ptn.mpo_average(p, h), ptn.mps_norm(p), ptn.mpo_average(p, mz),
                ptn.mpo_average(p, mx), ptn.mps_vdot(psi0, p)]

    fp = [fingerprint(psi)]
    nrms = []
    t0 = time.perf_counter()
    for k in range(numsteps):
        nrms.append(ptn.tdvp_singlesite(h, psi, dt, 1, numiter_lanczos=m))
        fp.append(fingerprint(psi))
        print(f"step {k + 1}: E={fp[-1][0].real:.15f} |psi|={fp[-1][1]:.15f} "
              f"({time.perf_counter() - t0:.0f} s)", flush=True)
    fp = np.array(fp)
    save("tdvp_xxz_l64.npz", **pack_mpo("h_", h), **pack_mpo("mz_", mz), **pack_mpo("mx_", mx),
         seed=np.array(seed), bonds=np.array(b), dt=np.array(dt), numsteps=np.array(numsteps),
         m=np.array(m), raw_sum=raw_sum, raw_first=raw_first, nrms=np.array(nrms),
         energy=fp[:, 0], norm=fp[:, 1].real, obs_z=fp[:, 2], obs_x=fp[:, 3], overlap0=fp[:, 4])


GENERATORS = {"chain_ops": gen_chain_ops, "krylov": gen_krylov, "block_qr": gen_block_qr,
              "mpos": gen_mpos, "tdvp_readme": gen_tdvp_readme, "tdvp_qnum": gen_tdvp_qnum,
              "dmrg": gen_dmrg, "tdvp_xxz_bulk": gen_tdvp_xxz_bulk,
              "ising_imag": gen_ising_imag, "mps_random": gen_mps_random,
              "apply_mpo": gen_apply_mpo, "twosite": gen_twosite, "compress": gen_compress,
              "tdvp_xxz_l64": gen_tdvp_xxz_l64}

if __name__ == "__main__":
    # all fixtures, or only the ones named on the command line (the L=64 one runs
    # for a quarter of an hour on 8 cores and is made only when named)
    for name in (sys.argv[1:] or [g for g in GENERATORS if g != "tdvp_xxz_l64"]):
        GENERATORS[name]()
