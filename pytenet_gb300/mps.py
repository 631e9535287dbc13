"""
Matrix product state container with the interface of pytenet.MPS
(pytenet/mps.py:14-178, 292-301).

Site tensors are held as NumPy arrays between calls, exactly like the
reference, so user code that edits `psi.a[i]` in place keeps working; the
sweeps upload them to the GPU once per call and write the results back.
Gauge operations (orthonormalize) run on the GPU.
"""

import numpy as np

from .qnumber import enforce_qsparsity, qnumber_outer_sum

__all__ = ["MPS", "crandn"]


def crandn(size=None, rng=None):
    """Standard complex normal samples, (N(0,1) + i N(0,1)) / sqrt(2), with all
    real parts drawn before all imaginary parts (pytenet/util.py:10-17)."""
    if rng is None:
        rng = np.random.default_rng()
    re = rng.normal(size=size)
    im = rng.normal(size=size)
    return (re + 1j * im) / np.sqrt(2)


class MPS:
    """MPS with site tensors of shape (b[i], d, b[i+1]) and integer quantum
    numbers `qsite` (physical) and `qbonds` (virtual), pytenet/mps.py:14-26."""

    def __init__(self, qsite, qbonds, fill=0.0, rng=None):
        """fill: scalar, "random" (complex Gaussian), "random real" or "postpone"
        (pytenet/mps.py:28-71)."""
        self.qsite = np.asarray(qsite)
        self.qbonds = [np.asarray(q) for q in qbonds]
        d = len(self.qsite)
        b = [len(q) for q in self.qbonds]
        assert b[0] == 1 and b[-1] == 1
        if isinstance(fill, (int, float, complex)) and not isinstance(fill, bool):
            self.a = [np.full((b[i], d, b[i + 1]), fill) for i in range(len(b) - 1)]
        elif fill == "random":
            if rng is None:
                rng = np.random.default_rng()
            self.a = [crandn((b[i], d, b[i + 1]), rng) / np.sqrt(b[i] * d * b[i + 1])
                      for i in range(len(b) - 1)]
        elif fill == "random real":
            if rng is None:
                rng = np.random.default_rng()
            self.a = [rng.normal(size=(b[i], d, b[i + 1])) / np.sqrt(b[i] * d * b[i + 1])
                      for i in range(len(b) - 1)]
        elif fill == "postpone":
            self.a = (len(b) - 1) * [None]
        else:
            raise ValueError(f'`fill` = {fill} invalid; must be a number, '
                             f'"random", "random real" or "postpone".')
        if fill != "postpone":
            for i, ai in enumerate(self.a):
                enforce_qsparsity(ai, [self.qbonds[i], self.qsite, -self.qbonds[i + 1]])

    @classmethod
    def construct_random(cls, nsites, qsite, qnum_sector, max_vdim=256, dtype="complex", rng=None):
        """Random MPS in a quantum-number sector with bonds capped at max_vdim; the
        random bond quantum numbers and entries are drawn in the reference's order
        (pytenet/mps.py:73-113)."""
        assert nsites > 0
        qsite = np.asarray(qsite)
        if rng is None:
            rng = np.random.default_rng()
        qb = (nsites + 1) * [None]
        qb[0] = [0]
        qb[-1] = [qnum_sector]

        def pick(full):
            if len(full) <= max_vdim:
                return full
            return full[rng.choice(len(full), size=max_vdim, replace=False)]

        for k in range(1, (nsites + 1) // 2):
            qb[k] = pick(qnumber_outer_sum([qb[k - 1], qsite]).reshape(-1))
        for k in reversed(range((nsites + 1) // 2, nsites)):
            qb[k] = pick(qnumber_outer_sum([qb[k + 1], -qsite]).reshape(-1))
        complex_entries = dtype in (complex, "complex")
        return cls(qsite, qb, fill=("random" if complex_entries else "random real"), rng=rng)

    @property
    def nsites(self):
        return len(self.a)

    @property
    def bond_dims(self):
        if len(self.a) == 0:
            return []
        return [x.shape[0] for x in self.a] + [self.a[-1].shape[2]]

    def zero_qnumbers(self):
        """Set all quantum numbers to zero (pytenet/mps.py:131-139)."""
        self.qsite.fill(0)
        for q in self.qbonds:
            q.fill(0)
        return self

    def orthonormalize(self, mode="left"):
        """Left or right QR orthonormalisation on the GPU; returns the norm
        (pytenet/mps.py:141-178)."""
        from .engine import DeviceMPS
        if len(self.a) == 0:
            return 1
        if mode not in ("left", "right"):
            raise ValueError(f'`mode` = {mode} invalid; must be "left" or "right".')
        dev = DeviceMPS(self)
        nrm = dev.orthonormalize(mode)
        dev.download(self)
        return float(nrm.item())

    def compress(self, tol, mode="svd", direction="left"):
        """Compress and orthonormalise on the GPU, by site-local truncated SVDs
        (mode "svd", pytenet/mps.py:180-236) or by rounding with local density
        matrices (mode "density", right to left, pytenet/mps.py:238-290); returns
        the original norm and the scaling factor of the compression."""
        if mode == "svd":
            from .compression import compress_svd
            return compress_svd(self, tol, direction)
        if mode == "density":
            from .compression import compress_density
            return compress_density(self, tol)
        raise ValueError(f'`mode` = {mode} invalid; must be "svd" or "density".')

    def to_vector(self):
        """Dense vector on the full Hilbert space (pytenet/mps.py:292-301); meant
        for small systems, used as the exact reference in checks."""
        v = self.a[0]
        for x in self.a[1:]:
            v = np.tensordot(v, x, axes=(2, 0))
            v = v.reshape((v.shape[0], v.shape[1] * v.shape[2], v.shape[3]))
        assert v.ndim == 3 and v.shape[0] == 1 and v.shape[2] == 1
        return v.reshape(-1)

    as_vector = to_vector
