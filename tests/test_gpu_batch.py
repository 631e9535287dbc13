"""Batched TDVP over independent instances: equal to the single-instance runs
(bitwise: same kernels and launch shapes, only the streams differ), against the
oracle, and with the autotuner's knobs."""

import copy
import warnings

import numpy as np
import pytest

from oracle import ptn_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ptg():
    import pytenet_gb300 as m
    from pytenet_gb300 import _lib
    _lib.load()
    return m


def small_batch(ptg, count=6, seed=21):
    from pytenet_gb300 import batch
    return batch.ising_batch(count, seed, lengths=(6, 10), dcaps=(4, 8, 16))


def clone(psi, ptg):
    p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
    p.a = [x.copy() for x in psi.a]
    return p


def test_batch_equals_single_runs_bitwise(ptg):
    hs, psis, _ = small_batch(ptg)
    singles = [clone(p, ptg) for p in psis]
    batched = [clone(p, ptg) for p in psis]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        nb = ptg.tdvp_singlesite_batch(hs, batched, 0.05, 3, numiter_lanczos=6, streams=3)
        ns = [ptg.tdvp_singlesite(h, p, 0.05, 3, numiter_lanczos=6) for h, p in zip(hs, singles)]
    assert nb == ns
    for pb, ps in zip(batched, singles):
        for x, y in zip(pb.a, ps.a):
            assert np.array_equal(x, y)


def test_batch_matches_oracle(ptg):
    hs, psis, _ = small_batch(ptg, count=5, seed=22)
    ref = [clone(p, ptg) for p in psis]
    out = [clone(p, ptg) for p in psis]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        norms = ptg.tdvp_singlesite_batch(hs, out, 0.05, 2, numiter_lanczos=6, streams=2)
        for h, p, n in zip(hs, ref, norms):
            oh = copy.deepcopy(h)
            nref = orc.tdvp_singlesite(oh, p, 0.05, 2, 6)
            assert abs(nref - n) < 1e-12
    for po, pr, h in zip(out, ref, hs):
        v, vr = orc.mps_to_vector(po), orc.mps_to_vector(pr)
        # imaginary time: compare the (unnormalised) states and their energies
        assert np.linalg.norm(v - vr) < 1e-10 * np.linalg.norm(vr)
        assert abs(orc.mpo_average(po, h) - orc.mpo_average(pr, h)) < 1e-10 * len(h.a)


def test_autotuned_batch(ptg):
    from pytenet_gb300 import autotune
    hs, psis, _ = small_batch(ptg, count=6, seed=23)
    a = [clone(p, ptg) for p in psis]
    b = [clone(p, ptg) for p in psis]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        t = autotune.tune_batch(hs, a, 6, "mixed")
        assert t["streams"] in autotune.STREAM_CANDIDATES
        cands = {str(k): v for k, v in autotune.CANDIDATES.items()}
        for vals in t["buckets"].values():
            for k, v in vals.items():
                assert v in cands[k] or v == autotune.DEFAULT_KNOBS.get(int(k) if k.isdigit() else k)
        ptg.tdvp_singlesite_batch(hs, a, 0.05, 2, numiter_lanczos=6, precision="mixed",
                                  autotune=True)
        ptg.tdvp_singlesite_batch(hs, b, 0.05, 2, numiter_lanczos=6, precision="mixed", streams=4)
    for pa, pb in zip(a, b):
        va, vb = orc.mps_to_vector(pa), orc.mps_to_vector(pb)
        assert np.linalg.norm(va - vb) < 1e-12 * np.linalg.norm(vb)
