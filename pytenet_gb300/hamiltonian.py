"""
Hamiltonians of the workloads as MPOs (host-side input generators, no GPU work).

Same operators as pytenet.heisenberg_xxz_1d_mpo (pytenet/hamiltonian/heisenberg.py:14-54)
and pytenet.ising_1d_mpo (pytenet/hamiltonian/ising.py:14-69). The reference builds
them through its operator-graph compiler (out of scope here); this module writes
the standard finite-automaton MPO directly and, for XXZ, merges the two channels
next to each chain end that carry multiples of the same end operator, which gives
the reference's bond dimensions (1, 4, 5, ..., 5, 4, 1). The tensors differ from
the reference's by the order and basis of the virtual states; the operator is the
same (identical to_matrix()), so every sweep result agrees. The reference's own
MPO objects can be passed to the sweeps as well.
"""

import numpy as np

from .mpo import MPO

__all__ = ["heisenberg_xxz_1d_mpo", "ising_1d_mpo"]


def _chain_mpo(qsite, qbond, bulk, nsites, start, end):
    """MPO from one bulk tensor (chi, d, d, chi): the first site keeps row
    `start`, the last site column `end`."""
    a = []
    for i in range(nsites):
        w = bulk
        if i == 0:
            w = w[start:start + 1]
        if i == nsites - 1:
            w = w[:, :, :, end:end + 1]
        a.append(np.array(w))
    qb = [np.array([qbond[start]])] + [np.array(qbond) for _ in range(nsites - 1)] + \
         [np.array([qbond[end]])]
    return MPO.from_tensors(qsite, qb, a)


def heisenberg_xxz_1d_mpo(nsites, J, D, h):
    """H = sum_i J (X_i X_{i+1} + Y_i Y_{i+1}) + D Z_i Z_{i+1} - h Z_i with spin-1/2
    operators (so J(XX+YY) = J/2 (S+S- + S-S+)), quantum numbers 2*Sz."""
    qsite = [1, -1]
    sup = np.array([[0., 1.], [0., 0.]])
    sdn = np.array([[0., 0.], [1., 0.]])
    sz = np.array([[0.5, 0.], [0., -0.5]])
    eye = np.identity(2)
    # automaton states: 0 nothing placed yet, 1 S+ open, 2 S- open, 3 Sz open, 4 done
    w = np.zeros((5, 2, 2, 5))
    w[0, :, :, 0] = eye
    w[0, :, :, 1] = sup
    w[0, :, :, 2] = sdn
    w[0, :, :, 3] = sz
    w[0, :, :, 4] = -h * sz
    w[1, :, :, 4] = 0.5 * J * sdn
    w[2, :, :, 4] = 0.5 * J * sup
    w[3, :, :, 4] = D * sz
    w[4, :, :, 4] = eye
    # MPO quantum-number rule q_a + q_out - q_in - q_b = 0: S+ raises by 2
    op = _chain_mpo(qsite, [0, 2, -2, 0, 0], w, nsites, 0, 4)
    a = [np.array(x) for x in op.a]
    qb = [np.array(q) for q in op.qbonds]
    if nsites >= 2:
        # first bond: "Sz open" (3) carries Sz_0 and "done" (4) carries -h Sz_0: one
        # channel carrying Sz_0, continued on site 1 by (row 3) - h (row 4)
        a[0] = a[0][:, :, :, :4]
        a[1] = np.concatenate([a[1][:3], a[1][3:4] - h * a[1][4:5]], axis=0)
        qb[1] = qb[1][:4]
    if nsites >= 3:
        # last bond: "nothing placed" (0) ends in -h Sz and "Sz open" (3) in D Sz: one
        # channel ending in Sz, entered from site L-2 through D (column 3) - h (column 0)
        m = D * a[-2][..., 3:4] - h * a[-2][..., 0:1]
        a[-2] = np.concatenate([m, a[-2][..., 1:3], a[-2][..., 4:5]], axis=3)
        last = np.zeros((4,) + a[-1].shape[1:])
        last[0, :, :, 0] = sz
        last[1:3] = a[-1][1:3]
        last[3] = a[-1][4]
        a[-1] = last
        qb[-2] = np.array([0, 2, -2, 0])
    return MPO.from_tensors(qsite, qb, a)


def ising_1d_mpo(nsites, J, h, g):
    """H = sum_i J Z_i Z_{i+1} + h Z_i + g X_i with Pauli matrices, zero quantum numbers."""
    qsite = [0, 0]
    sx = np.array([[0., 1.], [1., 0.]])
    sz = np.array([[1., 0.], [0., -1.]])
    eye = np.identity(2)
    # automaton states: 0 nothing placed, 1 Z open, 2 done
    w = np.zeros((3, 2, 2, 3))
    w[0, :, :, 0] = eye
    w[0, :, :, 1] = J * sz
    w[0, :, :, 2] = h * sz + g * sx
    w[1, :, :, 2] = sz
    w[2, :, :, 2] = eye
    return _chain_mpo(qsite, [0, 0, 0], w, nsites, 0, 2)
