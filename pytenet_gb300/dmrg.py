"""
Single-site DMRG on the GPU, drop-in for pytenet.dmrg_singlesite (pytenet/dmrg.py:22-93).
"""

import torch

from .device import device, to_host
from .engine import Chain, warn_breakdowns

__all__ = ["dmrg_singlesite"]


def dmrg_singlesite(hamiltonian, psi, numsweeps, numiter_lanczos=25, precision="fp64"):
    """Single-site DMRG; `psi` is overwritten with the optimised state; returns
    the energy after each sweep (pytenet/dmrg.py:22-93)."""
    nsites = len(hamiltonian.a)
    assert nsites == len(psi.a)
    chain = Chain(hamiltonian, psi, numiter_lanczos, precision)
    chain.orthonormalize("right")
    chain.init_envs()
    chain.check_envs()
    en = torch.zeros(numsweeps, dtype=torch.float64, device=device())
    for k in range(numsweeps):
        chain.dmrg_sweep(en, k)
    chain.download(psi)
    warn_breakdowns(chain)
    return to_host(en)
