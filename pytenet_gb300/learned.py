"""
Learned Lanczos depth for the TDVP local steps.

A 12 -> 64 -> 64 -> 1 FP32 MLP with GELU activations predicts, per local step,
how many Lanczos iterations reach a target accuracy. Inputs (computed on the
device after the first Lanczos iteration): site position, log2 bond dimensions,
step kind (site / bond), log10 |dt| |H v0|, and |dt| alpha_0..3, |dt| beta_0..2
of the previous run at the same site. At the predicted depth the run evaluates
the a-posteriori estimate beta_m |e_m^T exp(dt T_m) e_1| / |v| on the device and
stops there if it is below the tolerance; otherwise it continues to the full
depth (the fixed-depth method of pytenet/krylov.py:122-136).

Everything numerical runs in the library's kernels: feature extraction,
inference, the residual test, label computation and training (forward, backward
and Adam, ptn_mlp_*). This module only drives them.

Training data: TDVP runs at full depth in "record" mode log the features and the
whole tridiagonal matrix of every local step; the label is the smallest depth
whose residual estimate meets the tolerance (ptn_depth_labels).
"""

import os

import numpy as np
import torch

from . import _lib
from .device import call, device, lib, ptr, stream_ptr

__all__ = ["DepthModel", "collect_records", "labels", "features", "DEFAULT_WEIGHTS"]

M_SCALE = 20.0      # targets are depth / 20
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                               "depth_mlp.npz")


class DepthModel:
    """MLP parameters on the device plus Adam moments."""

    def __init__(self, params=None, seed=0):
        L = lib()
        self.n = L.ptn_mlp_param_count()
        if params is None:
            params = self.init_params(seed)
        params = np.asarray(params, dtype=np.float32)
        assert params.shape == (self.n,)
        self.params = torch.from_numpy(params.copy()).to(device())
        self.m = torch.zeros(self.n, dtype=torch.float32, device=device())
        self.v = torch.zeros(self.n, dtype=torch.float32, device=device())
        self.grad = torch.zeros(self.n, dtype=torch.float32, device=device())
        self.loss = torch.zeros(1, dtype=torch.float32, device=device())
        self.step = 0

    @staticmethod
    def init_params(seed=0):
        """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases; layout
        W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3."""
        rng = np.random.default_rng(seed)
        w1 = rng.uniform(-1, 1, (64, 12)) / np.sqrt(12)
        w2 = rng.uniform(-1, 1, (64, 64)) / np.sqrt(64)
        w3 = rng.uniform(-1, 1, 64) / np.sqrt(64)
        return np.concatenate([w1.ravel(), np.zeros(64), w2.ravel(), np.zeros(64), w3,
                               [0.4]]).astype(np.float32)

    # ------------------------------------------------------------ device ops
    def forward(self, X):
        X = torch.as_tensor(X, dtype=torch.float32, device=device()).contiguous()
        Y = torch.empty(X.shape[0], dtype=torch.float32, device=device())
        call(lib().ptn_mlp_forward, ptr(self.params), ptr(X), X.shape[0], ptr(Y), stream_ptr())
        return Y

    def gradient(self, X, T):
        """Mean-squared-loss gradient on the device; returns (grad, loss) tensors."""
        X = torch.as_tensor(X, dtype=torch.float32, device=device()).contiguous()
        T = torch.as_tensor(T, dtype=torch.float32, device=device()).contiguous()
        B = X.shape[0]
        L = lib()
        wsb = L.ptn_mlp_workspace_bytes(B)
        ws = torch.empty(wsb, dtype=torch.uint8, device=device())
        call(L.ptn_mlp_grad, ptr(self.params), ptr(X), ptr(T), B, ptr(self.grad), ptr(self.loss),
             ptr(ws), wsb, stream_ptr())
        return self.grad, self.loss

    def train(self, X, depth, epochs=200, batch=4096, lr=2e-3, seed=0, verbose=False):
        """Fit depth labels (integers) with minibatch Adam, all on the device."""
        X = torch.as_tensor(X, dtype=torch.float32, device=device()).contiguous()
        T = torch.as_tensor(np.asarray(depth, dtype=np.float32) / M_SCALE, device=device())
        n = X.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        L = lib()
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g).to(device())
            for s in range(0, n, batch):
                idx = perm[s:s + batch]
                self.gradient(X[idx], T[idx])
                self.step += 1
                call(L.ptn_mlp_adam, ptr(self.params), ptr(self.grad), ptr(self.m), ptr(self.v),
                     lr, 0.9, 0.999, 1e-8, self.step, stream_ptr())
            if verbose and (ep % 20 == 0 or ep == epochs - 1):
                hist.append(float(self.loss.item()))
                print(f"epoch {ep}: loss {hist[-1]:.5f}")
        return hist

    def predict_depth(self, X):
        y = self.forward(X).cpu().numpy()
        return np.maximum(np.ceil(y * M_SCALE).astype(int) + 1, 2)

    # ------------------------------------------------------------ persistence
    def save(self, path):
        np.savez_compressed(path, params=self.params.cpu().numpy())

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        return cls(np.load(path)["params"])


def collect_records(hamiltonian, psi, dt, numsteps, numiter=20, precision="mixed",
                    capacity=200000):
    """Run TDVP at full depth `numiter` in record mode; returns the device
    records (one row of _lib.DEPTH_RECORD doubles per local step)."""
    from .tdvp import TDVPRun
    run = TDVPRun(hamiltonian, psi, numiter_lanczos=numiter, precision=precision,
                  record_capacity=capacity)
    for _ in range(numsteps):
        run.step(dt)
    return run.chain.depth.records().clone()


def labels(records, m_max=20, tol=1e-10):
    """Smallest depth meeting the residual tolerance, per record (on the device)."""
    rec = records.contiguous()
    out = torch.empty(rec.shape[0], dtype=torch.int32, device=device())
    call(lib().ptn_depth_labels, ptr(rec), rec.shape[0], m_max, tol, ptr(out), stream_ptr())
    return out


def features(records):
    return records[:, :12].to(torch.float32).contiguous()
