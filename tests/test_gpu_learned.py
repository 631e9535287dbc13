"""Learned Lanczos depth: MLP forward / gradient kernels against the NumPy
checker, device labels against the CPU label rule, training, and the gain of
the trained network over the fixed-depth method at unchanged accuracy."""

import warnings

import numpy as np
import pytest

from oracle import mlp_oracle, ptn_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ptg():
    import pytenet_gb300 as m
    from pytenet_gb300 import _lib
    _lib.load()
    return m


def test_mlp_forward_and_gradient_match_oracle(ptg):
    from pytenet_gb300 import learned
    rng = np.random.default_rng(5)
    p = learned.DepthModel.init_params(3) + rng.normal(0, 0.05, 5057).astype(np.float32)
    X = rng.normal(size=(300, 12)).astype(np.float32)
    T = rng.uniform(0, 1, 300).astype(np.float32)
    model = learned.DepthModel(p)
    y = model.forward(X).cpu().numpy()
    y_ref = mlp_oracle.mlp_forward(p, X.astype(np.float64))
    assert np.max(np.abs(y - y_ref)) < 1e-5 * max(1.0, np.max(np.abs(y_ref)))
    g, loss = model.gradient(X, T)
    g_ref, loss_ref = mlp_oracle.mlp_grad(p, X.astype(np.float64), T.astype(np.float64))
    g = g.cpu().numpy()
    assert np.linalg.norm(g - g_ref) < 1e-4 * np.linalg.norm(g_ref)
    assert abs(float(loss.item()) - loss_ref) < 1e-5 * loss_ref


def _records(ptg, L=14, D=16, steps=2, seed=2):
    from pytenet_gb300 import learned
    rng = np.random.default_rng(seed)
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.9, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return learned.collect_records(h, psi, 0.05j, steps, precision="fp64", capacity=4096)


def test_depth_labels_match_cpu_rule(ptg):
    from pytenet_gb300 import learned
    rec = _records(ptg)
    lab = learned.labels(rec).cpu().numpy()
    R = rec.cpu().numpy()
    ref = np.array([mlp_oracle.depth_label(r) for r in R])
    assert len(lab) == 2 * (2 * 14 - 1) + 2 * (14 - 1) * 2   # site + bond steps per TDVP step
    # identical except possibly at estimates within rounding of the tolerance
    assert np.mean(lab == ref) > 0.98 and np.max(np.abs(lab - ref)) <= 1


def test_training_lowers_loss(ptg):
    from pytenet_gb300 import learned
    rec = _records(ptg, steps=3)
    lab = learned.labels(rec).cpu().numpy()
    X = learned.features(rec)
    model = learned.DepthModel(seed=4)
    _, l0 = model.gradient(X, lab / 20.0)
    l0 = float(l0.item())
    model.train(X, lab, epochs=150, batch=64, lr=3e-3)
    _, l1 = model.gradient(X, lab / 20.0)
    assert float(l1.item()) < 0.3 * l0


def test_learned_depth_saves_iterations_at_same_accuracy(ptg):
    """The trained network against the fixed-depth method it falls back to and
    against the residual criterion alone (the same a-posteriori estimate tested
    after every iteration from depth 2, no network): Lanczos iterations (operator
    applies) and the state against the fixed-depth run. Both early-exit forms must
    keep the state to 1e-10; the numbers of all three are printed."""
    import os
    from pytenet_gb300 import learned
    if os.path.exists(learned.DEFAULT_WEIGHTS):
        model = learned.DepthModel.load()
    else:
        rec = _records(ptg, L=20, D=32, steps=3)
        model = learned.DepthModel(seed=1)
        model.train(learned.features(rec), learned.labels(rec).cpu().numpy(), epochs=200, batch=128)
    rng = np.random.default_rng(11)
    L, D, numiter = 24, 32, 16
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 1.1, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    runs = {}
    for name, dm in (("fixed", None), ("residual", "residual"), ("learned", model)):
        p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
        p.a = [x.copy() for x in psi.a]
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            run = ptg.TDVPRun(h, p, numiter_lanczos=numiter, precision="fp64", depth_model=dm)
            for _ in range(3):
                run.step(0.05j)
        run.download()
        st = run.chain.krylov_state()
        runs[name] = (p, st.iters_total, st.early_exits)
    pf, itf, _ = runs["fixed"]
    ef = orc.mpo_average(pf, h).real
    for name in ("residual", "learned"):
        pl, itl, exits = runs[name]
        ov = orc.mps_vdot(pf, pl)
        infid = 1 - abs(ov) ** 2 / (orc.mps_vdot(pf, pf).real * orc.mps_vdot(pl, pl).real)
        el = orc.mpo_average(pl, h).real
        print(f"{name}: iterations {itl} (fixed {itf}), early exits {exits}, "
              f"infidelity {infid:.2e}, energy error {abs(ef - el):.2e}")
        assert exits > 0 and itl < 0.9 * itf
        assert infid < 1e-10
        assert abs(ef - el) < 1e-9 * max(1.0, abs(ef))
