"""
Matrix product operator container with the interface of pytenet.MPO
(pytenet/mpo.py:15-185, 225-235). The sweeps read the tensors once and keep a
complex128 copy on the GPU for the whole run.
"""

import numpy as np

from .mps import crandn
from .qnumber import enforce_qsparsity

__all__ = ["MPO"]


class MPO:
    """MPO with site tensors of shape (b[i], d, d, b[i+1]) and integer quantum
    numbers (pytenet/mpo.py:15-29)."""

    def __init__(self, qsite, qbonds, fill=0.0, rng=None):
        self.qsite = np.array(qsite)
        self.qbonds = [np.array(q) for q in qbonds]
        d = len(self.qsite)
        b = [len(q) for q in self.qbonds]
        if isinstance(fill, (int, float, complex)) and not isinstance(fill, bool):
            self.a = [np.full((b[i], d, d, b[i + 1]), fill) for i in range(len(b) - 1)]
        elif fill == "random":
            if rng is None:
                rng = np.random.default_rng()
            self.a = [crandn((b[i], d, d, b[i + 1]), rng) / np.sqrt(b[i] * d * b[i + 1])
                      for i in range(len(b) - 1)]
        elif fill == "random real":
            if rng is None:
                rng = np.random.default_rng()
            self.a = [rng.normal(size=(b[i], d, d, b[i + 1])) / np.sqrt(b[i] * d * b[i + 1])
                      for i in range(len(b) - 1)]
        elif fill == "postpone":
            self.a = (len(b) - 1) * [None]
        else:
            raise ValueError(f'`fill` = {fill} invalid; must be a number, '
                             f'"random", "random real" or "postpone".')
        if fill != "postpone":
            for i, ai in enumerate(self.a):
                enforce_qsparsity(ai, (self.qbonds[i], self.qsite, -self.qsite, -self.qbonds[i + 1]))

    @classmethod
    def from_tensors(cls, qsite, qbonds, tensors):
        """MPO from explicit site tensors (e.g. those of a reference pytenet.MPO)."""
        op = cls(qsite, qbonds, fill="postpone")
        op.a = [np.asarray(t) for t in tensors]
        return op

    @property
    def nsites(self):
        return len(self.a)

    @property
    def bond_dims(self):
        if len(self.a) == 0:
            return []
        return [x.shape[0] for x in self.a] + [self.a[-1].shape[3]]

    def zero_qnumbers(self):
        """Set all quantum numbers to zero (pytenet/mpo.py:177-185)."""
        self.qsite.fill(0)
        for q in self.qbonds:
            q.fill(0)
        return self

    def to_matrix(self):
        """Dense operator on the full Hilbert space (pytenet/mpo.py:225-235); for
        small systems, as the exact reference in checks."""
        m = self.a[0]
        for x in self.a[1:]:
            # m[b0, O, I, c] x[c, o, i, b2] -> [b0, (O, o), (I, i), b2]
            t = np.tensordot(m, x, axes=(3, 0))            # b0, O, I, o, i, b2
            t = t.transpose((0, 1, 3, 2, 4, 5))
            s = t.shape
            m = t.reshape((s[0], s[1] * s[2], s[3] * s[4], s[5]))
        assert m.shape[0] == 1 and m.shape[3] == 1
        return m.reshape((m.shape[1], m.shape[2]))

    as_matrix = to_matrix
