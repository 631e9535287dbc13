"""
Autotuner for the batched driver: per (bond-dimension bucket, d, chi) of the
batch, the library's launch-shape knobs (ptn_tune_set), and the number of CUDA
streams the batch is spread over.

Knobs (include/pytenet_gb300.h), plus "mmb", the smallest bond on which the mixed form
uses the tensor cores (a tensor-core GEMM CTA takes a whole SM's shared memory and
tensor memory, so in a batch small problems may overlap better on the FP64 path):
  PTN_TUNE_TC_SPLIT_WAVES    split-K target of the tensor-core digit GEMM
  PTN_TUNE_ZGEMM_SPLIT_WAVES split-K target of the FP64 GEMM
  PTN_TUNE_LARFB_TILE        block-update tile of the QR
  PTN_TUNE_QR_CLUSTER        cluster size cap of the QR panel
Each bucket is tuned on its most expensive instance by coordinate descent: one
knob at a time over its candidates, the others held, each candidate timed with
CUDA events over a time step of COPIES concurrent copies of that instance on as
many streams (graph replay after an eager and a captured step): in a batch the
kernels share the GPU, so a launch shape that fills every SM alone (deep split-K)
is not what is best there. The stream count is then chosen by timing batch steps
of a cost-ordered subset of the batch.
Results are cached per process (and, if PTN_TUNE_CACHE names a file, there as
JSON); knob values only change launch shapes, never the arithmetic of a kernel,
so tuned and untuned runs give results equal to rounding of the split-K sums.
"""

import contextlib
import json
import os

import numpy as np
import torch

from . import _lib
from .device import lib

__all__ = ["tune_batch", "knobs_for", "bucket_of", "DEFAULT_KNOBS"]

DEFAULT_KNOBS = {_lib.TUNE_TC_SPLIT_WAVES: 1, _lib.TUNE_ZGEMM_SPLIT_WAVES: 2,
                 _lib.TUNE_LARFB_TILE: 0, _lib.TUNE_QR_CLUSTER: 0, "mmb": 32}
CANDIDATES = {"mmb": [32, 64, 128, 1 << 20],
              _lib.TUNE_TC_SPLIT_WAVES: [0, 2],
              _lib.TUNE_ZGEMM_SPLIT_WAVES: [0, 2],
              _lib.TUNE_LARFB_TILE: [0, 1],
              _lib.TUNE_QR_CLUSTER: [0, 1]}
STREAM_CANDIDATES = [4, 8, 16]
COPIES = 4
_CACHE = {}


def bucket_of(psi, chi=None):
    """(largest bond dimension rounded up to a power of two, d, chi)."""
    dmax = max(max(a.shape[0], a.shape[2]) for a in psi.a)
    b = 1
    while b < dmax:
        b *= 2
    d = psi.a[0].shape[1]
    return (b, d, chi)


@contextlib.contextmanager
def knobs(values):
    """Set the library knobs of `values` (keys that are knob numbers) for the block."""
    L = lib()
    values = {k: v for k, v in values.items() if str(k).isdigit()}
    old = {int(k): L.ptn_tune_get(int(k)) for k in values}
    try:
        for k, v in values.items():
            _lib.check(L.ptn_tune_set(int(k), int(v)))
        yield
    finally:
        for k, v in old.items():
            L.ptn_tune_set(int(k), int(v))


def bucket_values(tuning, psi):
    """Tuned values of psi's bucket ({} without tuning)."""
    if not tuning:
        return {}
    return tuning["buckets"].get(str(bucket_of(psi)[:2]), {})


def knobs_for(tuning, psi):
    """Context setting the tuned knobs of psi's bucket (no-op without tuning)."""
    vals = bucket_values(tuning, psi)
    return knobs(vals) if vals else contextlib.nullcontext()


def _time_step(h, psi, numiter, precision, values, dt):
    from .batch import BatchTDVP
    b = BatchTDVP([h] * COPIES, [psi] * COPIES, numiter, precision, streams=COPIES, graph=True,
                  tuning={"buckets": {str(bucket_of(psi)[:2]): values}})
    b.step(dt)   # eager, captures the graphs
    b.step(dt)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    b.step(dt)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _tune_bucket(h, psi, numiter, precision, dt):
    best = {str(k): v for k, v in DEFAULT_KNOBS.items()}
    keys = [str(k) for k in CANDIDATES]
    if precision == "fp64":
        keys = [k for k in keys if k not in (str(_lib.TUNE_TC_SPLIT_WAVES), "mmb")]
    cands = {str(k): v for k, v in CANDIDATES.items()}
    t_best = _time_step(h, psi, numiter, precision, best, dt)
    trials = {json.dumps(best, sort_keys=True): t_best}
    for k in keys:
        for v in cands[k]:
            cand = dict(best)
            cand[k] = v
            key = json.dumps(cand, sort_keys=True)
            if key not in trials:
                trials[key] = _time_step(h, psi, numiter, precision, cand, dt)
            if trials[key] < t_best:
                best, t_best = cand, trials[key]
    return best, t_best


def tune_batch(hamiltonians, psis, numiter_lanczos, precision, dt=0.05, subset=16):
    """Knobs per bucket and the stream count for this batch (cached)."""
    from .batch import BatchTDVP, instance_cost
    sig = (tuple(sorted({bucket_of(p)[:2] for p in psis})), numiter_lanczos, precision)
    key = json.dumps(sig)
    path = os.environ.get("PTN_TUNE_CACHE")
    if key not in _CACHE and path and os.path.exists(path):
        with open(path) as f:
            _CACHE.update(json.load(f))
    if key in _CACHE:
        return _CACHE[key]
    buckets = {}
    for b in sorted({bucket_of(p)[:2] for p in psis}):
        idx = max((i for i, p in enumerate(psis) if bucket_of(p)[:2] == b),
                  key=lambda i: instance_cost(psis[i]))
        vals, _ = _tune_bucket(hamiltonians[idx], psis[idx], numiter_lanczos, precision, dt)
        buckets[str(b)] = {str(k): int(v) for k, v in vals.items()}
    tuning = {"buckets": buckets, "streams": 8}
    # streams: batch steps of a subset spread like the whole batch
    order = sorted(range(len(psis)), key=lambda i: -instance_cost(psis[i]))
    sub = order[::max(1, len(order) // subset)][:subset]
    times = {}
    for s in STREAM_CANDIDATES:
        if s > len(sub):
            continue
        b = BatchTDVP([hamiltonians[i] for i in sub], [psis[i] for i in sub], numiter_lanczos,
                      precision, streams=s, graph=True, tuning=tuning)
        b.step(dt)   # eager, captures the graphs
        b.step(dt)   # first replay
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        b.step(dt)
        e1.record()
        torch.cuda.synchronize()
        times[str(s)] = e0.elapsed_time(e1)
        del b
    if times:
        tuning["streams"] = int(min(times, key=lambda s: (times[s], int(s))))
    tuning["stream_times_ms"] = times
    _CACHE[key] = tuning
    if path:
        with open(path, "w") as f:
            json.dump(_CACHE, f)
    return tuning
