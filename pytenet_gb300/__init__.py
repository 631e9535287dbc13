"""
pytenet_gb300 -- GB300-native engine for PyTeNet's single-site TDVP / DMRG sweeps.

Drop-in API of the reference package (cmendl/pytenet) for this path:
    tdvp_singlesite, dmrg_singlesite, MPS, MPO,
    apply_local_hamiltonian, apply_local_bond_contraction,
    contraction_operator_step_left / _right, compute_right_operator_blocks,
    lanczos_iteration, expm_krylov, eigh_krylov, eigh_tridiag,
    block_sparse_qr and the quantum-number helpers,
    heisenberg_xxz_1d_mpo, ising_1d_mpo, mpo_average, mps_vdot, mps_norm, apply_mpo;
and, next to the single-site path, tdvp_twosite / dmrg_twosite with
block_sparse_svd, split_block_sparse_matrix_svd and retained_bond_indices.
Additions: TDVPRun (device-resident run, optional CUDA graph), BatchTDVP /
tdvp_singlesite_batch (many independent instances on streams), the mixed
precision form (precision="mixed") and the learned Lanczos depth (learned.py).

All numerics run in hand-written CUDA kernels for sm_103a (libptn_gb300.so,
C ABI in include/pytenet_gb300.h). There is no CPU fallback: without the
library or a GPU the compute functions raise.
"""

from .mps import MPS, crandn
from .mpo import MPO
from .qnumber import (qnumber_outer_sum, qnumber_flatten, common_qnumbers, is_qsparse,
                      enforce_qsparsity, sort_by_qnumbers)
from .hamiltonian import heisenberg_xxz_1d_mpo, ising_1d_mpo
from .block_sparse import block_sparse_qr, block_sparse_svd, split_block_sparse_matrix_svd
from .bond_ops import retained_bond_indices
from .chain_ops import (apply_local_hamiltonian, apply_local_bond_contraction,
                        contraction_operator_step_left, contraction_operator_step_right,
                        compute_right_operator_blocks, mpo_average, mpo_inner_product,
                        mps_vdot, mps_norm, apply_mpo)
from .krylov import lanczos_iteration, expm_krylov, eigh_krylov, eigh_tridiag
from .tdvp import tdvp_singlesite, TDVPRun
from .dmrg import dmrg_singlesite
from .twosite import tdvp_twosite, dmrg_twosite, merge_mpo_pair
from .batch import BatchTDVP, tdvp_singlesite_batch
from ._lib import PtnError, PtnShapeError

__version__ = "0.1.0"
