"""
Batched single-site TDVP: many independent MPS instances (different lengths,
bond dimensions and couplings) advanced together on one GPU.

Each instance is a device-resident TDVPRun (pytenet/tdvp.py:26-118 per instance,
the same kernels and the same results as running it alone). The batch is spread
over S CUDA streams by a greedy bin-pack on the instances' cost
(sum over sites of Dl Dr (Dl + Dr)), longest first, so that the many small
kernels of different instances run side by side and fill the 152 SMs. After one
eager step per instance, every instance's time step is captured once as a CUDA
graph; a batch time step is then one graph launch per instance, issued
round-robin into the streams (a single graph over the whole batch would hold
millions of kernel nodes).

The schedule (S, and the per-bucket tuning knobs of the library: split-K wave
targets of the FP64 and tensor-core GEMMs, block-update tiles of the QR) comes
from autotune.tune_batch when `autotune=True`, otherwise from defaults.
"""

import warnings

import numpy as np
import torch

from . import _lib
from .tdvp import TDVPRun

__all__ = ["BatchTDVP", "tdvp_singlesite_batch", "instance_cost", "assign_streams"]


def instance_cost(psi):
    """Relative work of one TDVP step of an instance: sum over sites of Dl Dr (Dl + Dr)."""
    c = 0.0
    for a in psi.a:
        Dl, _, Dr = a.shape
        c += float(Dl) * Dr * (Dl + Dr)
    return c


def assign_streams(costs, nstreams):
    """Greedy longest-processing-time bin-pack of instance costs onto streams;
    returns a list of instance-index lists, one per stream (deterministic)."""
    nstreams = max(1, min(int(nstreams), len(costs)))
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * nstreams
    groups = [[] for _ in range(nstreams)]
    for i in order:
        k = min(range(nstreams), key=lambda s: (loads[s], s))
        groups[k].append(i)
        loads[k] += costs[i]
    return groups


class BatchTDVP:
    """Device-resident batch of TDVP runs.

    hamiltonians, psis: lists of MPO / MPS (psis are overwritten by download()).
    streams: number of CUDA streams (None: from the tuner or 8).
    graph: capture each instance's step as a CUDA graph after its first step.
    autotune / tuning: run autotune.tune_batch first, or use its result."""

    def __init__(self, hamiltonians, psis, numiter_lanczos=25, precision="fp64", streams=None,
                 graph=True, autotune=False, tuning=None):
        assert len(hamiltonians) == len(psis) and len(psis) > 0
        self.psis = psis
        self.precision = precision
        self.tuning = tuning
        if autotune and tuning is None:
            from .autotune import tune_batch
            self.tuning = tune_batch(hamiltonians, psis, numiter_lanczos, precision)
            if streams is None:
                streams = self.tuning["streams"]
        self.nstreams = int(streams) if streams is not None else 8
        self.costs = [instance_cost(p) for p in psis]
        self.groups = assign_streams(self.costs, self.nstreams)
        self.streams = [torch.cuda.Stream() for _ in self.groups]
        self.runs = [None] * len(psis)
        main = torch.cuda.current_stream()
        for k, grp in enumerate(self.groups):
            self.streams[k].wait_stream(main)
            with torch.cuda.stream(self.streams[k]):
                for i in grp:
                    with self._knobs(psis[i]):
                        self.runs[i] = TDVPRun(hamiltonians[i], psis[i], numiter_lanczos,
                                               precision, graph=graph,
                                               mixed_min_bond=self._mixed_min_bond(psis[i]))
        for s in self.streams:
            main.wait_stream(s)
        self.steps_done = 0

    def _knobs(self, psi):
        """The tuned knobs of psi's bucket, and the three-launch Lanczos step: the
        instances run concurrently on several streams, and the fused step's grid
        barriers assume the whole GPU."""
        from .autotune import bucket_values, knobs
        vals = dict(bucket_values(self.tuning, psi))
        vals[str(_lib.TUNE_KRYLOV_FUSED)] = 0
        return knobs(vals)

    def _mixed_min_bond(self, psi):
        from .autotune import bucket_values
        v = bucket_values(self.tuning, psi).get("mmb")
        return None if v is None else int(v)

    def step(self, dt, capture=True):
        """Exactly one time step of every instance (capture: record each
        instance's CUDA graph at its first step, for the following ones)."""
        main = torch.cuda.current_stream()
        for s in self.streams:
            s.wait_stream(main)
        for k, grp in enumerate(self.groups):
            with torch.cuda.stream(self.streams[k]):
                for i in grp:
                    with self._knobs(self.psis[i]):
                        self.runs[i].step(dt, capture)
        for s in self.streams:
            main.wait_stream(s)
        self.steps_done += 1

    def norms(self):
        """Norms of the initial states (what tdvp_singlesite returns per instance)."""
        return [float(r.nrm.item()) for r in self.runs]

    def download(self):
        torch.cuda.synchronize()
        for r in self.runs:
            r.download()
        return self.psis

    def breakdowns(self):
        return sum(r.chain.breakdowns() for r in self.runs)


def tdvp_singlesite_batch(hamiltonians, psis, dt, numsteps, numiter_lanczos=25, precision="fp64",
                          streams=None, graph=True, autotune=False, tuning=None):
    """tdvp_singlesite over a list of independent instances; every psi is
    overwritten in place and the list of initial norms is returned."""
    b = BatchTDVP(hamiltonians, psis, numiter_lanczos, precision, streams, graph, autotune,
                  tuning)
    for n in range(numsteps):
        b.step(dt, capture=(n < numsteps - 1))
    b.download()
    nb = b.breakdowns()
    if nb:
        warnings.warn(f"Lanczos iteration stopped early (beta ~= 0) in {nb} local step(s) "
                      f"across the batch.", RuntimeWarning, stacklevel=2)
    return b.norms()


def random_product_state(qsite, nsites, dcap, rng):
    """Seeded random product state embedded at bond dimensions
    min(2^min(i, L - i), dcap): site tensors are zero except [0, :, 0], a normalised
    complex Gaussian vector per site (drawn site by site)."""
    from .mps import MPS
    d = len(qsite)
    bonds = [min(2 ** min(i, nsites - i), dcap) for i in range(nsites + 1)]
    psi = MPS(qsite, [b * [0] for b in bonds], fill="postpone")
    tensors = []
    for i in range(nsites):
        a = np.zeros((bonds[i], d, bonds[i + 1]), dtype=complex)
        v = rng.normal(size=d) + 1j * rng.normal(size=d)
        a[0, :, 0] = v / np.linalg.norm(v)
        tensors.append(a)
    psi.a = tensors
    return psi


def ising_batch(count, seed, lengths=(16, 48), dcaps=(32, 64, 128, 256)):
    """The batch workload: `count` transverse-field Ising chains, J = 1,
    g ~ U[0.5, 1.5], h ~ U[0, 0.2], L ~ U{lengths}, bond cap drawn from dcaps,
    random product initial states (all draws from one seeded generator)."""
    from .hamiltonian import ising_1d_mpo
    rng = np.random.default_rng(seed)
    hs, psis, meta = [], [], []
    for _ in range(count):
        L = int(rng.integers(lengths[0], lengths[1] + 1))
        dcap = int(dcaps[int(rng.integers(0, len(dcaps)))])
        g = float(rng.uniform(0.5, 1.5))
        h = float(rng.uniform(0.0, 0.2))
        H = ising_1d_mpo(L, 1.0, h, g)
        hs.append(H)
        psis.append(random_product_state(H.qsite, L, dcap, rng))
        meta.append({"L": L, "D": dcap, "g": g, "h": h})
    return hs, psis, meta
