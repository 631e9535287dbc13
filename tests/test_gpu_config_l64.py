"""The plain complex128 form at scale against the reference: XXZ L=64 (J=1,
Delta=0.8, h=-0.1, zero quantum numbers), bonds min(2^min(i, L-i), 256), seeded
complex Gaussian entries, left-orthonormalised, real time dt=0.05j, 20 steps of
tdvp_singlesite with numiter_lanczos=10.

The fixture tests/golden/tdvp_xxz_l64.npz holds what the reference itself
computed on this input (tests/golden/gen_golden.py tdvp_xxz_l64, one call of the
reference's tdvp_singlesite per step): its MPO tensors and, after every step,
gauge-invariant fingerprints of the state -- energy, norm, the returned norm, two
weighted one-site observables sum_i c_i <Sz_i> and sum_i c'_i <Sx_i> and the
overlap with the initial state. The 134 MB state is regenerated here from the
seed; the draw order is the reference's (checked against stored checksums)."""

import numpy as np
import pytest

from conftest import golden_mpo, load_golden

pytestmark = pytest.mark.gpu


def test_tdvp_xxz_l64_d256_matches_reference():
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    from pytenet_gb300.chain_ops import mpo_average, mps_norm, mps_vdot
    _lib.load()
    g = load_golden("tdvp_xxz_l64.npz")
    h, mz, mx = golden_mpo(g, "h_"), golden_mpo(g, "mz_"), golden_mpo(g, "mx_")
    L, dt, m = len(h.a), complex(g["dt"]), int(g["m"])
    rng = np.random.default_rng(int(g["seed"]))
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in g["bonds"]], fill="random", rng=rng)
    # the same draws as the reference's MPS(..., fill="random"), bit for bit
    assert np.array_equal(np.array([x.sum() for x in psi.a]), g["raw_sum"])
    assert np.array_equal(np.array([x.reshape(-1)[0] for x in psi.a]), g["raw_first"])
    psi.orthonormalize(mode="left")
    psi0 = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
    psi0.a = [x.copy() for x in psi.a]

    def fingerprint(p):
        return [mpo_average(p, h), mps_norm(p), mpo_average(p, mz), mpo_average(p, mx),
                mps_vdot(psi0, p)]

    fp = [fingerprint(psi)]
    nrms = []
    for _ in range(int(g["numsteps"])):
        nrms.append(ptg.tdvp_singlesite(h, psi, dt, 1, numiter_lanczos=m))
        fp.append(fingerprint(psi))
    fp = np.array(fp)
    dE = np.abs(fp[:, 0] - g["energy"])
    dn = np.abs(fp[:, 1].real - g["norm"])
    dz = np.abs(fp[:, 2] - g["obs_z"])
    dx = np.abs(fp[:, 3] - g["obs_x"])
    dov = np.abs(fp[:, 4] - g["overlap0"])
    dnrm = np.abs(np.array(nrms) - g["nrms"])
    print("max deviations per quantity over the 21 states:",
          f"energy {dE.max():.2e} (rel {(dE / np.abs(g['energy'])).max():.2e}),",
          f"norm {dn.max():.2e}, Sz {dz.max():.2e}, Sx {dx.max():.2e},",
          f"overlap {dov.max():.2e}, returned norm {dnrm.max():.2e}")
    # relative 1e-10 on every gauge-invariant quantity of every step
    assert (dE <= 1e-10 * np.abs(g["energy"])).all(), dE
    assert (dn <= 1e-10 * g["norm"]).all(), dn
    assert (dnrm <= 1e-10 * np.abs(g["nrms"])).all(), dnrm
    assert (dz <= 1e-10 * np.maximum(np.abs(g["obs_z"]), 1e-3)).all(), dz
    assert (dx <= 1e-10 * np.maximum(np.abs(g["obs_x"]), 1e-3)).all(), dx
    assert (dov <= 1e-10 * np.abs(g["overlap0"])).all(), dov
