"""
Bond truncation rule of the two-site splits (pytenet/bond_ops.py:23-38): host-side
integer bookkeeping on the singular values the device computed.
"""

import numpy as np

__all__ = ["retained_bond_indices"]


def retained_bond_indices(s, tol):
    """Indices of the singular values kept at tolerance `tol`: the normalised squares
    s_i^2 / |s|^2, accumulated from the smallest value up, must exceed tol. An
    all-zero spectrum keeps nothing (pytenet/bond_ops.py:23-38)."""
    s = np.asarray(s, dtype=float)
    w = np.linalg.norm(s)
    if w == 0:
        return np.array([], dtype=int)
    sq = (s / w) ** 2
    order = np.argsort(sq)
    acc = np.empty_like(sq)
    acc[order] = np.cumsum(sq[order])
    return np.where(acc > tol)[0]
