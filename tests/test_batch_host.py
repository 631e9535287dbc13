"""Host logic of the batched driver and the tuning knobs (no GPU needed)."""

import numpy as np
import pytest

from pytenet_gb300 import batch


def test_assign_streams_is_a_balanced_deterministic_partition():
    rng = np.random.default_rng(0)
    costs = list(rng.uniform(1, 100, 57))
    g1 = batch.assign_streams(costs, 8)
    g2 = batch.assign_streams(costs, 8)
    assert g1 == g2
    assert sorted(i for g in g1 for i in g) == list(range(57))
    loads = [sum(costs[i] for i in g) for g in g1]
    # longest-processing-time bound: max load <= mean + largest item
    assert max(loads) <= np.mean(loads) + max(costs)
    assert batch.assign_streams([1.0, 2.0], 8) == [[1], [0]]


def test_ising_batch_workload_draws():
    hs, psis, meta = batch.ising_batch(12, seed=5)
    hs2, psis2, meta2 = batch.ising_batch(12, seed=5)
    assert meta == meta2
    for h, p, m in zip(hs, psis, meta):
        assert 16 <= m["L"] <= 48 and m["D"] in (32, 64, 128, 256)
        assert 0.5 <= m["g"] <= 1.5 and 0.0 <= m["h"] <= 0.2
        assert len(h.a) == m["L"] == len(p.a)
        bonds = [a.shape[0] for a in p.a] + [p.a[-1].shape[2]]
        assert bonds == [min(2 ** min(i, m["L"] - i), m["D"]) for i in range(m["L"] + 1)]
        for a in p.a:
            # product state: only [0, :, 0] is non-zero, normalised
            assert abs(np.linalg.norm(a[0, :, 0]) - 1) < 1e-14
            assert np.count_nonzero(a) <= a.shape[1]
    costs = [batch.instance_cost(p) for p in psis]
    assert all(c > 0 for c in costs)


def test_tuning_knobs_validate_and_round_trip():
    from pytenet_gb300 import _lib
    L = _lib.load()
    for k, v in ((_lib.TUNE_TC_SPLIT_WAVES, 4), (_lib.TUNE_ZGEMM_SPLIT_WAVES, 0),
                 (_lib.TUNE_LARFB_TILE, 3)):
        old = L.ptn_tune_get(k)
        assert L.ptn_tune_set(k, v) == _lib.PTN_OK and L.ptn_tune_get(k) == v
        assert L.ptn_tune_set(k, old) == _lib.PTN_OK
    assert L.ptn_tune_set(_lib.TUNE_LARFB_TILE, 9) == _lib.PTN_BAD_SHAPE
    assert L.ptn_tune_set(_lib.TUNE_QR_PANEL, 4) == _lib.PTN_BAD_SHAPE
    assert L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, 2) == _lib.PTN_BAD_SHAPE
    assert L.ptn_tune_get(_lib.TUNE_QR_PANEL) == 0 and L.ptn_tune_get(_lib.TUNE_TC_PERSISTENT) == 0
    assert L.ptn_tune_set(8, 1) == _lib.PTN_BAD_SHAPE
    assert L.ptn_tune_get(_lib.TUNE_TC_SKIP_ZERO) == 0
    assert L.ptn_tune_get(_lib.TUNE_TC_SPLIT_WAVES) == 1


def test_tuner_buckets_and_knob_context():
    from pytenet_gb300 import _lib, autotune
    L = _lib.load()
    _, psis, meta = batch.ising_batch(6, seed=3)
    for p, m in zip(psis, meta):
        b, d, _ = autotune.bucket_of(p)
        assert d == 2 and b >= max(max(a.shape[0], a.shape[2]) for a in p.a) and b & (b - 1) == 0
    tuning = {"buckets": {str(autotune.bucket_of(psis[0])[:2]):
                          {str(_lib.TUNE_LARFB_TILE): 3, str(_lib.TUNE_QR_CLUSTER): 1, "mmb": 64}}}
    vals = autotune.bucket_values(tuning, psis[0])
    assert vals["mmb"] == 64
    before = (L.ptn_tune_get(_lib.TUNE_LARFB_TILE), L.ptn_tune_get(_lib.TUNE_QR_CLUSTER))
    with autotune.knobs_for(tuning, psis[0]):
        assert L.ptn_tune_get(_lib.TUNE_LARFB_TILE) == 3
        assert L.ptn_tune_get(_lib.TUNE_QR_CLUSTER) == 1
    assert (L.ptn_tune_get(_lib.TUNE_LARFB_TILE), L.ptn_tune_get(_lib.TUNE_QR_CLUSTER)) == before
    assert autotune.bucket_values(None, psis[0]) == {}
