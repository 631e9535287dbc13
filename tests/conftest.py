import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


class _Obj:
    pass


def golden_mps(g, prefix):
    """Rebuild an MPS-like object (a, qsite, qbonds) stored by gen_golden.py."""
    n = int(g[prefix + "n"])
    o = _Obj()
    o.qsite = g[prefix + "qsite"].copy()
    o.a = [g[f"{prefix}a{i}"].copy() for i in range(n)]
    o.qbonds = [g[f"{prefix}qb{i}"].copy() for i in range(n + 1)]
    o.nsites = n
    return o


def golden_mpo(g, prefix):
    n = int(g[prefix + "n"])
    o = _Obj()
    o.qsite = g[prefix + "qsite"].copy()
    o.a = [g[f"{prefix}w{i}"].copy() for i in range(n)]
    o.qbonds = [g[f"{prefix}qb{i}"].copy() for i in range(n + 1)]
    o.nsites = n
    return o


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
