"""
Quantum-number bookkeeping of the block-sparse tensors: exact integer work on the
host, with the semantics of pytenet/block_sparse_util.py:13-103.

The numerical part of block_sparse_qr runs on the device (block_sparse.py); this
module decides, from the integer quantum numbers alone, which rows and columns
form each block, in which order the blocks are stacked and which quantum numbers
the new bond carries. Those decisions depend only on integers, so a whole sweep
can be planned ahead of its numerics.
"""

import numpy as np

__all__ = ["qnumber_outer_sum", "qnumber_flatten", "common_qnumbers", "is_qsparse",
           "enforce_qsparsity", "sort_by_qnumbers", "QRPlan", "qr_plan"]


def qnumber_outer_sum(qnums):
    """All sums of one entry from each list, as a tensor
    (pytenet/block_sparse_util.py:13-30)."""
    if len(qnums) == 0:
        return np.array(0)
    t = np.asarray(qnums[0])
    for q in qnums[1:]:
        t = np.add.outer(t, np.asarray(q))
    return t


def qnumber_flatten(qnums):
    """Flattened outer sum (pytenet/block_sparse_util.py:40-44)."""
    return qnumber_outer_sum(qnums).reshape(-1)


def common_qnumbers(qnums0, qnums1):
    """Sorted common values (pytenet/block_sparse_util.py:33-37)."""
    return np.intersect1d(qnums0, qnums1)


def is_qsparse(a, qnums):
    """Whether every entry with a non-zero quantum-number sum vanishes
    (pytenet/block_sparse_util.py:47-53). Accepts NumPy arrays or device tensors."""
    mask = qnumber_outer_sum(qnums) != 0
    if not mask.any():
        return True   # no entry is constrained (e.g. all quantum numbers zero)
    if hasattr(a, "is_cuda"):
        import torch
        m = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(mask, tuple(a.shape))))
        return not bool(torch.any((a != 0) & m.to(a.device)).item())
    a = np.asarray(a)
    return not np.any(np.where(mask, a, 0))


def enforce_qsparsity(a, qnums):
    """Zero every entry with a non-zero quantum-number sum, in place
    (pytenet/block_sparse_util.py:56-64)."""
    mask = qnumber_outer_sum(qnums) != 0
    a[np.broadcast_to(mask, a.shape)] = 0


def sort_by_qnumbers(a, q0, q1):
    """Stable sort of rows / columns by quantum number
    (pytenet/block_sparse_util.py:67-92)."""
    q0 = np.asarray(q0)
    q1 = np.asarray(q1)
    idx0 = np.argsort(q0, kind="mergesort")
    idx1 = np.argsort(q1, kind="mergesort")
    if np.any(idx0 - np.arange(len(idx0))):
        q0 = q0[idx0]
        a = a[idx0, :]
    if np.any(idx1 - np.arange(len(idx1))):
        q1 = q1[idx1]
        a = a[:, idx1]
    return a, (idx0, q0), (idx1, q1)


class QRPlan:
    """Integer plan of one block_sparse_qr call.

    blocks: list of (rows, cols, k0, kb): original row / column indices of the
            block (in sorted order), and its column range [k0, k0+kb) in Q.
    K:      new bond dimension; qinterm: its quantum numbers.
    dense:  single block covering all rows and columns in original order (the
            zero-quantum-number case): no gather / scatter is needed.
    empty:  no common quantum number (pytenet/block_sparse_util.py:124-135).
    """

    def __init__(self, q0, q1):
        q0 = np.asarray(q0)
        q1 = np.asarray(q1)
        self.m, self.n = len(q0), len(q1)
        qis = common_qnumbers(q0, q1)
        self.blocks = []
        if len(qis) == 0:
            self.empty = True
            self.dense = False
            self.K = 1
            self.qinterm = q0[:1].copy()
            return
        self.empty = False
        idx0 = np.argsort(q0, kind="mergesort")
        idx1 = np.argsort(q1, kind="mergesort")
        s0, s1 = q0[idx0], q1[idx1]
        k = 0
        qint = []
        for qn in qis:
            r = np.where(s0 == qn)[0]
            c = np.where(s1 == qn)[0]
            rows = idx0[r[0]:r[-1] + 1]
            cols = idx1[c[0]:c[-1] + 1]
            kb = min(len(rows), len(cols))
            self.blocks.append((rows.astype(np.int64), cols.astype(np.int64), k, kb))
            qint.append(np.full(kb, qn, dtype=q0.dtype))
            k += kb
        self.K = k
        self.qinterm = np.concatenate(qint)
        self.dense = (len(self.blocks) == 1 and len(self.blocks[0][0]) == self.m
                      and len(self.blocks[0][1]) == self.n
                      and np.array_equal(self.blocks[0][0], np.arange(self.m))
                      and np.array_equal(self.blocks[0][1], np.arange(self.n)))
        self.dev_cache = {}


_PLANS = {}


def qr_plan(q0, q1):
    """Cached QRPlan for the quantum numbers of rows (q0) and columns (q1)."""
    q0 = np.ascontiguousarray(q0)
    q1 = np.ascontiguousarray(q1)
    key = (q0.dtype.str, q0.tobytes(), q1.dtype.str, q1.tobytes())
    p = _PLANS.get(key)
    if p is None:
        if len(_PLANS) > 4096:
            _PLANS.clear()
        p = QRPlan(q0, q1)
        _PLANS[key] = p
    return p
