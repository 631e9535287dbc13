"""
Train the learned Lanczos-depth MLP on the GPU and write
pytenet_gb300/data/depth_mlp.npz.

Training data are full-depth (20 iterations) TDVP runs in record mode on
synthetic workloads of the two families the model is used on:
  - XXZ chains L=64 (J=1, h=-0.1, Delta ~ U[0.5, 1.5] per run, seeded), bond caps
    D in {32, 64, 128, 256, 512}, real time dt=0.05j;
  - transverse-field Ising chains (J=1, g ~ U[0.5, 1.5], h ~ U[0, 0.2]), L in
    {16..48}, D in {32, 64, 128}, imaginary time dt=0.05.
Labels: smallest depth whose residual estimate is <= 1e-10 (ptn_depth_labels).
Collection, labels, training and evaluation all run in the library's kernels.

    python -m pytenet_gb300.train_depth [--out PATH] [--quick]
"""

import argparse
import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import pytenet_gb300 as ptg  # noqa: E402
from pytenet_gb300 import learned  # noqa: E402


def xxz_state(L, D, rng, delta):
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, delta, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    return h, psi


def ising_state(L, D, rng):
    g, hz = rng.uniform(0.5, 1.5), rng.uniform(0.0, 0.2)
    h = ptg.ising_1d_mpo(L, 1.0, hz, g)
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    return h, psi


def collect(quick=False, seed=7):
    rng = np.random.default_rng(seed)
    recs = []
    plan_xxz = [(32, 12), (64, 8), (128, 4), (256, 2), (512, 1)]
    plan_ising = [(32, 4), (64, 3), (128, 2)]
    if quick:
        plan_xxz = [(16, 3), (32, 2)]
        plan_ising = [(16, 2)]
    for D, steps in plan_xxz:
        for _ in range(2 if not quick else 1):
            h, psi = xxz_state(64 if not quick else 24, D, rng, rng.uniform(0.5, 1.5))
            recs.append(learned.collect_records(h, psi, 0.05j, steps))
    for D, steps in plan_ising:
        for _ in range(4 if not quick else 1):
            L = int(rng.integers(16, 49)) if not quick else 16
            h, psi = ising_state(L, D, rng)
            recs.append(learned.collect_records(h, psi, 0.05, steps))
    return torch.cat(recs, 0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=learned.DEFAULT_WEIGHTS)
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--epochs", type=int, default=300)
    a = ap.parse_args()
    t0 = time.time()
    rec = collect(a.quick)
    lab = learned.labels(rec).cpu().numpy()
    X = learned.features(rec)
    n = X.shape[0]
    perm = np.random.default_rng(0).permutation(n)
    ntest = max(1, n // 10)
    te, tr = perm[:ntest], perm[ntest:]
    model = learned.DepthModel(seed=1)
    model.train(X[torch.as_tensor(tr, device=X.device)], lab[tr], epochs=a.epochs, verbose=True)
    pred = model.predict_depth(X[torch.as_tensor(te, device=X.device)])
    under = float(np.mean(pred < lab[te]))
    saved = float(np.mean(np.maximum(0, 20 - np.maximum(pred, lab[te]))))
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    model.save(a.out)
    summary = {"records": int(n), "label_hist": np.bincount(lab, minlength=21).tolist(),
               "test_underestimate_fraction": under, "test_mean_depth_saved_vs_20": saved,
               "seconds": time.time() - t0}
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
