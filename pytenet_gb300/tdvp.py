"""
Single-site TDVP on the GPU, drop-in for pytenet.tdvp_singlesite (pytenet/tdvp.py:26-118).
"""

import numpy as np
import torch

from .engine import Chain, warn_breakdowns

__all__ = ["tdvp_singlesite", "TDVPRun"]


class TDVPRun:
    """Device-resident TDVP run: upload once, step many times, download when
    asked. `tdvp_singlesite` is this class driven for `numsteps` steps.

    precision: "fp64" (plain complex128) or "mixed" (fixed-point BF16 digit
    contractions on the tensor cores, FP64 Krylov / QR).
    depth_model: a trained learned.DepthModel; numiter_lanczos is then the full
    depth the run falls back to whenever the residual estimate at the predicted
    depth exceeds depth_tol. depth_model="residual" tests the same estimate after
    every iteration from depth 2 on, with no network (the residual-only criterion).
    graph: capture one time step in a CUDA graph after the first step and
    replay it (all buffers are preallocated and no step synchronises).
    mixed_min_bond: smallest bond on which the mixed form uses the tensor cores
    (default engine.MIXED_MIN_BOND)."""

    def __init__(self, hamiltonian, psi, numiter_lanczos=25, precision="fp64", graph=False,
                 depth_model=None, depth_tol=1e-10, record_capacity=0, mixed_min_bond=None):
        nsites = len(hamiltonian.a)
        assert nsites == len(psi.a)
        self.psi = psi
        depth = None
        if depth_model is not None or record_capacity > 0:
            from .engine import DepthState
            residual = isinstance(depth_model, str)
            if residual and depth_model != "residual":
                raise ValueError('depth_model must be a DepthModel, "residual" or None')
            params = depth_model.params if (depth_model is not None and not residual) else None
            depth = DepthState(nsites, params, depth_tol, record_capacity,
                               check_from=2 if residual else 0)
        self.chain = Chain(hamiltonian, psi, numiter_lanczos, precision, depth=depth,
                           mixed_min_bond=mixed_min_bond)
        # right-normalise, build the environments (pytenet/tdvp.py:51-63)
        self.nrm = self.chain.orthonormalize("right").clone()
        self.chain.init_envs()
        self.chain.check_envs()
        self.use_graph = graph
        self.graph = None
        self.graph_dt = None
        self.steps_done = 0

    def _state_key(self):
        return ([q.tobytes() for q in self.chain.qbonds], list(self.chain.shape))

    def step(self, dt, capture=True):
        """Exactly one symmetric time step exp(-dt H) (pytenet/tdvp.py:65-115).
        With graph=True the first step runs eagerly and, if it left the integer
        state (shapes, quantum numbers) unchanged, the same step is captured as a
        CUDA graph -- capturing records without executing -- which later steps
        with the same dt replay. capture=False skips the capture (a last step)."""
        if self.graph is not None and self.graph_dt == dt:
            self.graph.replay()
            self.steps_done += 1
            return
        before = self._state_key()
        self.chain.tdvp_step(dt)
        self.steps_done += 1
        if self.use_graph and capture and self._state_key() == before:
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self.chain.tdvp_step(dt)
            torch.cuda.current_stream().wait_stream(s)
            assert self._state_key() == before
            self.graph = g
            self.graph_dt = dt

    def download(self):
        self.chain.download(self.psi)
        return self.psi

    # ------------------------------------------------ measurements on the device
    def tensors(self):
        """Current site tensors as device views (no copy)."""
        return [self.chain.site(i) for i in range(self.chain.nsites)]

    def energy(self):
        """<psi|H|psi> of the current state, contracted in FP64 on the device
        (pytenet/chain_ops.py:151-162 without the host round trip)."""
        from .chain_ops import mpo_average
        return mpo_average(self.tensors(), self.chain.w)

    def vdot(self, other):
        """<other|psi> against another run (or MPS / tensor list) of equal bonds."""
        from .chain_ops import mps_vdot
        o = other.tensors() if isinstance(other, TDVPRun) else other
        return mps_vdot(o, self.tensors())

    def norm(self):
        return float(np.sqrt(self.vdot(self).real))


def tdvp_singlesite(hamiltonian, psi, dt, numsteps, numiter_lanczos=25, precision="fp64",
                    graph=False, depth_model=None, depth_tol=1e-10):
    """Symmetric single-site TDVP; `psi` is overwritten in place with the evolved
    state and the norm of the initial `psi` is returned (pytenet/tdvp.py:26-118).
    All numerics run on the GPU."""
    run = TDVPRun(hamiltonian, psi, numiter_lanczos, precision, graph, depth_model, depth_tol)
    for n in range(numsteps):
        run.step(dt, capture=(n < numsteps - 1))
    run.download()
    warn_breakdowns(run.chain)
    return float(run.nrm.item())
