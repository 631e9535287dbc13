"""
Benchmark: single-site TDVP site-updates/s on the XXZ chain, L=64, D=512
(dt = 0.05j, numiter_lanczos = 10, Delta drawn uniformly in [0.5, 1.5] from a
seeded generator, zero quantum numbers, seeded complex Gaussian left-orthonormal
MPS with bonds min(2^min(i, L-i), D)).

One "step" is one symmetric TDVP time step = 2L-1 site updates. Inputs are
resident in HBM when the timed region starts; the whole state (site tensors,
environments, Krylov basis: several GB) is far larger than the 129 MB L2, so no
explicit L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form learned|mixed|fp64] [--no-graph]

Forms: "fp64" = complex128 everywhere, fixed Lanczos depth (the reference's
method); "mixed" = tensor-core contractions from five fixed-point BF16 digits per
row-scaled value (exact integer accumulation of the leading digit levels, FP64
recombination) with FP64 Krylov / QR, fixed depth; "learned" (default) = "mixed" plus the
learned Lanczos depth (trained MLP, residual-guarded early exit, falling back to the full
depth); "residual" = "mixed" with the same residual estimate tested after every iteration
from depth 2 and no network (the baseline the learned depth is measured against). Each timed step is replayed as a captured CUDA graph unless --no-graph.
  python bench.py --impl reference ...   # the reference CPU algorithm (NumPy restatement
                                         # pinned to the reference's outputs) on this host's
                                         # cores: whole time steps of the same chain
Other workloads (one JSON line each, not the headline):
  --workload xxz-d1024     XXZ L=32, D=1024: mixed TDVP against FP64 per step, and DMRG
  --workload ising-batch   256 independent Ising chains (add --autotune)
  --workload qr            ptn_qr (Q and R) of seeded complex 512x256, 1024x512 and
                           2048x1024 matrices for each QR kernel form, against LAPACK

Multi-GPU: the sweep does not shard (site i+1 depends on site i), so N GPUs run
N independent replicas of the workload (weak scaling, no collective on the data
path); value = total site updates / max-over-ranks time.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TDVP site-updates/s, XXZ L=64 D=512, mixed+learned vs FP64 plain at <=1e-8 E err"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--form", default=os.environ.get("PTN_BENCH_FORM", "learned"),
                   choices=["learned", "residual", "mixed", "fp64"])
    p.add_argument("--depth-tol", type=float, default=1e-10)
    p.add_argument("--tc-split-waves", type=int, default=None,
                   help="PTN_TUNE_TC_SPLIT_WAVES for the run (library default if unset)")
    p.add_argument("--tc-persistent", type=int, default=None, choices=[0, 1],
                   help="PTN_TUNE_TC_PERSISTENT for the run (library default if unset)")
    p.add_argument("--L", type=int, default=64)
    p.add_argument("--D", type=int, default=512)
    p.add_argument("--m", type=int, default=10)
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--e2e-steps", type=int, default=1)
    p.add_argument("--acc-steps", type=int, default=3,
                   help="steps of the mixed form in lockstep with the FP64 form (energy, "
                        "infidelity, norm drift after each; FP64 steps after the first are "
                        "timed for vs_fp64)")
    p.add_argument("--cpu-sites", type=int, default=3)
    p.add_argument("--ref-budget", type=float, default=150.0,
                   help="--impl reference: seconds of whole time steps to time (at least one)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-accuracy", action="store_true")
    p.add_argument("--no-graph", dest="graph", action="store_false",
                   help="launch every kernel eagerly instead of replaying each time step as a "
                        "captured CUDA graph")
    p.add_argument("--workload", default="xxz", choices=["xxz", "ising-batch", "xxz-d1024", "qr"])
    p.add_argument("--dmrg-sweeps", type=int, default=4)
    p.add_argument("--dmrg-acc-sweeps", type=int, default=1)
    p.add_argument("--batch-count", type=int, default=256)
    p.add_argument("--batch-seed", type=int, default=2027)
    p.add_argument("--streams", type=int, default=None)
    p.add_argument("--autotune", action="store_true")
    p.add_argument("--cpu-instances", type=int, default=2)
    p.add_argument("--qr-default-only", action="store_true",
                   help="--workload qr: only the default kernels on the 1024x512 matrix")
    a = p.parse_args()
    if a.steps is None:
        a.steps = 1 if (a.form == "fp64" or a.workload == "ising-batch") else 5
    assert a.warmup >= 3, "at least 3 warm-up steps"
    return a


def workload_desc(a):
    return (f"XXZ L={a.L} D={a.D} J=1 h=-0.1 Delta~U[0.5,1.5] (seed {a.seed}), "
            f"dt=0.05j, numiter_lanczos={a.m}, one step = 2L-1 site updates")


def make_workload(a, ptg_mod=None):
    """Host-side inputs (seeded). Returns (mpo, psi, Delta); psi is not yet
    orthonormalised."""
    rng = np.random.default_rng(a.seed)
    delta = float(rng.uniform(0.5, 1.5))
    if ptg_mod is not None:
        h = ptg_mod.heisenberg_xxz_1d_mpo(a.L, 1.0, delta, -0.1)
        h.zero_qnumbers()
        b = [min(2 ** min(i, a.L - i), a.D) for i in range(a.L + 1)]
        psi = ptg_mod.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
        return h, psi, delta
    from pytenet_gb300.hamiltonian import heisenberg_xxz_1d_mpo  # host-only module
    h = heisenberg_xxz_1d_mpo(a.L, 1.0, delta, -0.1)
    h.zero_qnumbers()
    return h, None, delta


# ------------------------------------------------------------------ CPU sample
def cpu_sample(a, nsites_sample, rng_seed=7):
    """Bounded sample of the same workload on the host cores with the NumPy
    restatement of the reference algorithm: `nsites_sample` bulk site updates
    (site expm with numiter applies, QR, left environment, bond expm, absorb) at
    bond D with random environments of the right shapes. Returns seconds per
    bulk site update and the sweep-average site-updates/s implied by the chain's
    bond profile (cost ~ D_l * D_r * max(D_l, D_r) per site)."""
    from oracle import ptn_oracle as orc
    h, _, _ = make_workload(a)
    D, d, m = a.D, 2, a.m
    rng = np.random.default_rng(rng_seed)
    w = h.a[a.L // 2]
    chi = w.shape[0]

    def herm_env():
        x = orc.crandn((D, chi, D), rng) / D
        return 0.5 * (x + x.conj().transpose(2, 1, 0))

    l, r = herm_env(), herm_env()
    aa = orc.crandn((D, d, D), rng)
    aa /= np.linalg.norm(aa)
    nxt = orc.crandn((D, d, D), rng)
    dt = 0.05j
    q0 = np.zeros(D * d, dtype=int)
    q1 = np.zeros(D, dtype=int)
    t0 = time.perf_counter()
    for _ in range(nsites_sample):
        x = orc._site_step(l, r, w, aa, 0.5 * dt, m)
        q, c, _ = orc.block_sparse_qr(x.reshape(D * d, D), q0, q1)
        x = q.reshape(D, d, D)
        ln = orc.env_step_left(x, x, w, l)
        c = orc._bond_step(ln, r, c, -0.5 * dt, m)
        _ = np.tensordot(c, nxt, (1, 0))
    sec = (time.perf_counter() - t0) / nsites_sample
    b = [min(2 ** min(i, a.L - i), a.D) for i in range(a.L + 1)]
    cost = [b[i] * b[i + 1] * max(b[i], b[i + 1]) for i in range(a.L)]
    weights = np.array(cost, float) / float(D ** 3)
    # L-1 sites in each direction plus the last site once: every site twice but one
    sweep_units = 2.0 * weights.sum() - weights[-1]
    sweep_sec = sweep_units * sec
    return sec, (2 * a.L - 1) / sweep_sec


def reference_arm(a):
    """--impl reference: the reference's CPU algorithm -- the NumPy restatement of
    pytenet's tdvp_singlesite, pinned to outputs of the reference itself -- on this
    host's cores, same workload, metric and config as our arm. Set-up (right
    normalisation, right environments) is untimed; every timed step is one whole
    symmetric TDVP time step (2L-1 site updates) of the L=64 chain. Whole steps
    take about a minute and a half each on 16 cores, so the arm times as many as
    fit in --ref-budget seconds (at least one), and prints exactly that count."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import warnings
    from oracle import ptn_oracle as orc
    cores = os.cpu_count()
    h, _, delta = make_workload(a)
    rng = np.random.default_rng(a.seed)
    rng.uniform(0.5, 1.5)   # the Delta draw of make_workload
    b = [min(2 ** min(i, a.L - i), a.D) for i in range(a.L + 1)]
    psi = orc.random_mps(h.qsite, [np.zeros(bi, dtype=int) for bi in b], rng)
    orc.orthonormalize(psi, mode="left")
    t_setup = time.perf_counter()
    _, lblocks, rblocks = orc.tdvp_setup(h, psi)
    t_setup = time.perf_counter() - t_setup
    # warm-up: BLAS threads and allocator on bulk-sized local steps (the sweep's
    # state is not touched)
    wrng = np.random.default_rng(7)
    w = h.a[a.L // 2]
    for _ in range(a.warmup):
        x = orc.crandn((a.D, 2, a.D), wrng)
        env = orc.crandn((a.D, w.shape[0], a.D), wrng)
        orc.apply_local_hamiltonian(x, w, env, env)
    dt = 0.05j
    secs = []
    t_all = time.perf_counter()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        while len(secs) < a.steps:
            t0 = time.perf_counter()
            orc.tdvp_step(h, psi, lblocks, rblocks, dt, a.m)
            secs.append(time.perf_counter() - t0)
            if time.perf_counter() - t_all + secs[-1] > a.ref_budget:
                break
    sec = float(np.mean(secs))
    value = (2 * a.L - 1) / sec
    sample = (f"{len(secs)} whole TDVP time step(s) of the L={a.L} D={a.D} chain "
              f"({2 * a.L - 1} site updates each) of the NumPy restatement of pytenet's "
              f"tdvp_singlesite, {cores} host cores; {len(secs)} of the {a.steps} requested "
              f"steps fit the {a.ref_budget:.0f} s budget; set-up (right normalisation and "
              f"environments, {t_setup:.1f} s) untimed")
    out = {"metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": a.gpus,
           "steps": len(secs), "requested_steps": a.steps, "warmup": a.warmup,
           "ms_per_step": sec * 1e3, "step_seconds": secs,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": workload_desc(a), "delta": delta,
                      "l2": "inputs larger than L2"},
           "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores,
                            "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ our arm
def max_over_ranks(ms, device):
    """Slowest rank's time (replicas run the same workload; the job takes as long
    as its slowest replica)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, site_updates, steps, ms_max):
    """Whole-job site-updates/s of `world` independent replicas (weak scaling)."""
    return world * site_updates * steps / (ms_max / 1e3)


def kern_key(form):
    return "zgemm_dmma" if form == "fp64" else "tc_gemm"


def capture_traffic(kernel, D):
    """Mean dram__bytes_read.sum + dram__bytes_write.sum per launch of `kernel` at
    bond D from the ncu capture summarised in profiles/traffic.json, or None."""
    try:
        rec = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        e = rec[kernel][str(D)]
        return float(e["bytes_per_launch"]), e["capture"]
    except Exception:
        return None, None


def krylov_roofline(ms, nbytes, launches, peaks):
    """Achieved HBM bandwidth of the fused Lanczos step (one cooperative launch per
    iteration: reads w, v_j, v_{j-1}, writes v_{j+1}; 64 bytes per vector entry)
    from the library's CUDA-event hooks, against the measured copy bandwidth."""
    if not launches or ms <= 0:
        return None
    peak = peaks.get("hbm_gbs", 6800.0)
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"kernel": "k_lanczos_fused", "bound": "hbm", "achieved": gbs, "peak": peak,
            "unit": "GB/s", "frac": gbs / peak, "launches": launches,
            "bytes_per_launch": nbytes / launches,
            "peak_source": "hbm_gbs of measured" if "hbm_gbs" in peaks else "hbm of fallback"}


def our_arm(a):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    L = _lib.load()

    if a.tc_split_waves is not None:
        _lib.check(L.ptn_tune_set(_lib.TUNE_TC_SPLIT_WAVES, a.tc_split_waves))
    if a.tc_persistent is not None:
        _lib.check(L.ptn_tune_set(_lib.TUNE_TC_PERSISTENT, a.tc_persistent))
    h, psi, delta = make_workload(a, ptg)
    psi.orthonormalize(mode="left")
    psi_host0 = [x.copy() for x in psi.a]
    qb0 = [q.copy() for q in psi.qbonds]
    site_updates = 2 * a.L - 1

    prec = "fp64" if a.form == "fp64" else "mixed"
    depth_model = None
    if a.form == "learned":
        from pytenet_gb300.learned import DepthModel
        depth_model = DepthModel.load()
    elif a.form == "residual":
        depth_model = "residual"
    run = ptg.TDVPRun(h, psi, numiter_lanczos=a.m, precision=prec, graph=a.graph,
                      depth_model=depth_model, depth_tol=a.depth_tol)
    dt = 0.05j
    for _ in range(a.warmup):
        run.step(dt)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = L.ptn_launch_count()
    dominant = 0 if a.form == "fp64" else 1
    ks0 = run.chain.krylov_state()
    L.ptn_prof_start((1 << dominant) | (1 << 3) | (1 << 4))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(a.steps):
        run.step(dt)
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    L.ptn_prof_stop()
    launches = L.ptn_launch_count() - launches0
    ks1 = run.chain.krylov_state()
    prof_from = "the timed steps"
    prof_ms = None   # time the profiled steps took
    if a.graph:
        # graph replays bypass the host-side launch hooks: kernel timings and the
        # launch count come from one further, eager step of the same run
        n0 = L.ptn_launch_count()
        L.ptn_prof_start((1 << dominant) | (1 << 3) | (1 << 4))
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        p0.record()
        run.chain.tdvp_step(dt)
        p1.record()
        torch.cuda.synchronize()
        L.ptn_prof_stop()
        prof_ms = p0.elapsed_time(p1)
        launches = (L.ptn_launch_count() - n0) * a.steps
        prof_from = "one eager step after the timed graph replays (same kernels and shapes)"
    nlocal = a.steps * (2 * a.L - 1 + 2 * (a.L - 1))
    krylov = {"local_steps": nlocal, "lanczos_iterations": ks1.iters_total - ks0.iters_total,
              "mean_depth": (ks1.iters_total - ks0.iters_total) / nlocal,
              "early_exits": ks1.early_exits - ks0.early_exits, "full_depth": a.m,
              "depth_tol": a.depth_tol if a.form in ("learned", "residual") else None}
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    if prof_ms is None:
        prof_ms = ms
    ms_max = max_over_ranks(ms, "cuda")
    value = replica_value(world, site_updates, a.steps, ms_max)

    def prof(kind):
        import ctypes
        tot, fl, by, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        _lib.check(L.ptn_prof_read(kind, ctypes.byref(tot), ctypes.byref(fl), ctypes.byref(by),
                                   ctypes.byref(n)))
        return tot.value, fl.value, by.value, n.value

    k_ms, k_fl, k_by, k_n = prof(dominant)
    q_ms, q_fl, q_by, q_n = prof(3)
    kr_ms, kr_fl, kr_by, kr_n = prof(4)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if dominant == 1:
        # the GEMM is timed inside seconds-long steps: the sustained BF16 figure
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        peak_src = ("bf16_tflops_sustained of measured" if "bf16_tflops_sustained" in peaks
                    else "bf16 sustained of fallback")
        achieved = k_fl / (k_ms / 1e3) / 1e12 if k_ms > 0 else None
        unit = "TFLOP/s"
        kern = "tcgen05 BF16-digit complex GEMM (5 digits)"
    else:
        # FP64 tensor (DMMA) peak: measured on this machine's GB300 with a DMMA-only kernel
        peak = 1.047
        peak_src = "FP64 DMMA m8n8k4 throughput measured on GB300 (1.047 TFLOP/s)"
        achieved = k_fl / (k_ms / 1e3) / 1e12 if k_ms > 0 else None
        unit = "TFLOP/s"
        kern = "DMMA complex128 GEMM"
    # DRAM bytes per launch of the dominant kernel: from one ncu capture of the same
    # kernel at the same bulk GEMM shapes, kept under profiles/ (null if none matches)
    traffic, traffic_src = capture_traffic(kern_key(a.form), a.D)
    roofline = {"bound": "tensor", "kernel": kern, "achieved": achieved, "peak": peak,
                "unit": unit, "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "traffic_unit": "bytes per launch" if traffic else None,
                "traffic_source": traffic_src,
                "digit_product_tflops": (achieved * 15.0) if (achieved and dominant == 1) else None,
                "peak_source": peak_src, "launches_timed": k_n,
                "kernel_share_of_step": (k_ms / prof_ms) if prof_ms > 0 else None,
                "qr_share_of_step": (q_ms / prof_ms) if prof_ms > 0 else None,
                "flops_per_launch": (k_fl / k_n) if k_n else None, "timings_from": prof_from,
                "krylov_step": krylov_roofline(kr_ms, kr_by, kr_n, peaks)}

    # ---- accuracy of the mixed form vs the FP64 form (same initial state), and
    # the FP64 form's own rate on the same chain
    accuracy, fp64 = None, None
    if a.form != "fp64" and not a.no_accuracy and rank == 0:
        accuracy, fp64 = accuracy_vs_fp64(a, ptg, h, psi_host0, qb0, depth_model)

    # ---- e2e through the public API with host buffers
    e2e = None
    if a.e2e_steps > 0:
        psi_e = ptg.MPS(psi.qsite, qb0, fill="postpone")
        psi_e.a = [x.copy() for x in psi_host0]
        h2d = sum(x.nbytes for x in psi_e.a) + sum(np.asarray(w, complex).nbytes for w in h.a)
        d2h = sum(x.nbytes for x in psi_e.a)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            ptg.tdvp_singlesite(h, psi_e, dt, 1, numiter_lanczos=a.m, precision=prec,
                                depth_model=depth_model, depth_tol=a.depth_tol)
        torch.cuda.synchronize()
        et = time.perf_counter() - t0
        e2e = {"value": world * site_updates * a.e2e_steps / et, "unit": "site-updates/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "steps": a.e2e_steps,
               "what": "tdvp_singlesite(hamiltonian, psi_host, dt, numsteps=1) per step: "
                       "upload, right-normalisation, environments, one step, download"}

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        sec, rate = cpu_sample(a, a.cpu_sites)
        cpu = {"value": rate, "unit": "site-updates/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{a.cpu_sites} bulk site updates at D={a.D} ({sec:.2f} s each) of the "
                         f"NumPy restatement of pytenet's tdvp_singlesite on all host cores; "
                         f"sweep-average rate from the chain's bond profile"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world,
               "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_max / a.steps,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "c128" if a.form == "fp64" else "bf16 digits (5 x 8-bit fixed point, tcgen05) + f64",
               "data": "synthetic",
               "config": {"workload": workload_desc(a), "form": a.form, "L": a.L, "D": a.D,
                          "numiter_lanczos": a.m, "delta": delta, "graph": a.graph,
                          "tc_split_waves": L.ptn_tune_get(_lib.TUNE_TC_SPLIT_WAVES),
                          "tc_persistent": L.ptn_tune_get(_lib.TUNE_TC_PERSISTENT),
                          "parallelism": f"replicas x{world}",
                          "l2": "inputs larger than L2 (state of several GB per replica)"},
               "krylov": krylov, "clocks": clk, "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline,
               "cpu_baseline": cpu, "accuracy_vs_fp64": accuracy,
               "fp64_value": fp64["value"] if fp64 else None,
               "vs_fp64": (value / world / fp64["value"]) if fp64 else None,
               "fp64_form": fp64}
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------------ batch workload
BATCH_METRIC = "TDVP site-updates/s, batch of 256 transverse-field Ising chains (L 16..48, D cap 32..256)"


def batch_desc(a):
    return (f"{a.batch_count} transverse-field Ising chains (seed {a.batch_seed}): J=1, "
            f"g~U[0.5,1.5], h~U[0,0.2], L~U{{16..48}}, D cap from {{32,64,128,256}}, random product "
            f"states embedded at the capped bonds; imaginary time dt=0.05, numiter_lanczos={a.m}; "
            f"one step = sum over instances of (2L-1) site updates")


def batch_cpu_sample(a, hs, psis, ninst):
    """NumPy restatement of pytenet's tdvp_singlesite on all host cores for one
    time step of `ninst` instances spread over the batch's cost range; the whole
    batch's CPU time is extrapolated by the instances' cost (sum Dl Dr (Dl + Dr))."""
    import copy
    from oracle import ptn_oracle as orc
    from pytenet_gb300.batch import instance_cost
    costs = np.array([instance_cost(p) for p in psis])
    order = np.argsort(costs)
    # cheapest quartile: a sample that stays within seconds on the host
    pick = [int(order[int(q * (len(order) - 1) * 0.25)]) for q in np.linspace(0.2, 1.0, ninst)]
    secs, cost = 0.0, 0.0
    import warnings
    for i in pick:
        p = copy.deepcopy(psis[i])
        t0 = time.perf_counter()
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            orc.tdvp_singlesite(copy.deepcopy(hs[i]), p, 0.05, 1, a.m)
        secs += time.perf_counter() - t0
        cost += costs[i]
    batch_sec = costs.sum() * secs / cost
    site_updates = sum(2 * len(h.a) - 1 for h in hs)
    sample = (f"one time step of {len(pick)} instances (L={[len(hs[i].a) for i in pick]}, "
              f"{secs:.1f} s) of the NumPy restatement; batch time extrapolated by instance cost")
    return site_updates / batch_sec, batch_sec, sample


def batch_arm(a):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib, batch
    L = _lib.load()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    hs, psis, meta = batch.ising_batch(a.batch_count, a.batch_seed)
    host0 = [[x.copy() for x in p.a] for p in psis]
    prec = "fp64" if a.form == "fp64" else "mixed"
    dt = 0.05
    site_updates = sum(2 * len(h.a) - 1 for h in hs)
    t_setup = time.perf_counter()
    b = ptg.BatchTDVP(hs, psis, a.m, prec, streams=a.streams, autotune=a.autotune)
    for _ in range(a.warmup):
        b.step(dt)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(a.steps):
        b.step(dt)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    value = site_updates * a.steps / (ms / 1e3)
    print(json.dumps({"partial": True, "value": value, "ms_per_step": ms / a.steps,
                      "tuning": b.tuning, "streams": b.nstreams}), file=sys.stderr, flush=True)
    # kernel split and launch count from one eager step of every instance (graph
    # replays bypass the host-side hooks), under each instance's tuned knobs
    import ctypes
    launches0 = L.ptn_launch_count()
    L.ptn_prof_start(0x1F)
    torch.cuda.synchronize()
    for p, r in zip(psis, b.runs):
        with b._knobs(p):
            r.chain.tdvp_step(dt)
    torch.cuda.synchronize()
    L.ptn_prof_stop()
    prof_note = "one eager step of every instance, instance order; the library's hooks keep " \
                "the first 32768 timed launches"
    launches_step = L.ptn_launch_count() - launches0
    kinds = {}
    for k, name in enumerate(["zgemm_dmma (FP64 GEMM)", "tc_gemm (tcgen05 digit GEMM)",
                              "mpo_stage", "qr", "krylov"]):
        tot, fl, by, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        _lib.check(L.ptn_prof_read(k, ctypes.byref(tot), ctypes.byref(fl), ctypes.byref(by),
                                   ctypes.byref(n)))
        kinds[name] = {"ms": tot.value, "flops": fl.value, "bytes": by.value, "launches": n.value}
    dom = "tc_gemm (tcgen05 digit GEMM)" if prec == "mixed" else "zgemm_dmma (FP64 GEMM)"
    kd = kinds[dom]
    achieved = kd["flops"] / (kd["ms"] / 1e3) / 1e12 if kd["ms"] > 0 else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0) if prec == "mixed" else 1.047
    eager_total = sum(v["ms"] for v in kinds.values())
    roofline = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak if achieved else None, "traffic": None,
                "peak_source": ("bf16_tflops of measured" if prec == "mixed" else
                                "FP64 DMMA m8n8k4 throughput measured on GB300 (1.047 TFLOP/s)"),
                "measured_on": prof_note,
                "kind_ms_eager_step": {k: v["ms"] for k, v in kinds.items()},
                "kind_share_eager_step": {k: (v["ms"] / eager_total if eager_total else None)
                                          for k, v in kinds.items()}}
    # e2e through the public API: host MPS in and out, one step
    e2e = None
    if a.e2e_steps > 0:
        pe = []
        for p, t in zip(psis, host0):
            q = ptg.MPS(p.qsite, p.qbonds, fill="postpone")
            q.a = [x.copy() for x in t]
            pe.append(q)
        h2d = sum(x.nbytes for q in pe for x in q.a) + sum(
            np.asarray(w, complex).nbytes for h in hs for w in h.a)
        d2h = sum(x.nbytes for q in pe for x in q.a)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ptg.tdvp_singlesite_batch(hs, pe, dt, a.e2e_steps, a.m, prec, streams=b.nstreams,
                                      graph=False, tuning=b.tuning)
        torch.cuda.synchronize()
        et = time.perf_counter() - t0
        e2e = {"value": site_updates * a.e2e_steps / et, "unit": "site-updates/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "steps": a.e2e_steps,
               "what": "tdvp_singlesite_batch(hs, psis_host, dt, numsteps) incl. uploads, "
                       "right-normalisation, environments, download"}
    cpu = None
    if not a.no_cpu:
        rate, bsec, sample = batch_cpu_sample(a, hs, [ptg_clone(ptg, p, t) for p, t in
                                                     zip(psis, host0)], a.cpu_instances)
        cpu = {"value": rate, "unit": "site-updates/s", "cores": os.cpu_count(), "kind": "port",
               "sample": sample}
    dmix = {}
    for m_ in meta:
        dmix[m_["D"]] = dmix.get(m_["D"], 0) + 1
    out = {"metric": BATCH_METRIC, "value": value, "unit": "site-updates/s", "n_gpus": 1,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "c128" if prec == "fp64" else "bf16 digits (5 x 8-bit fixed point, tcgen05) + f64",
           "data": "synthetic",
           "config": {"workload": batch_desc(a), "form": prec, "instances": a.batch_count,
                      "site_updates_per_step": site_updates, "d_caps": dmix,
                      "streams": b.nstreams, "autotune": bool(a.autotune), "graphs": True,
                      "tuning": b.tuning, "setup_and_warmup_s": t_setup,
                      "l2": "inputs larger than L2 (batch state of many GB)"},
           "clocks": clk, "e2e": e2e, "gpu_launches": int(launches_step * a.steps),
           "gpu_launches_note": "kernels per batch step counted on an eager step, times steps "
                                "(the timed steps replay captured graphs of them)",
           "roofline": roofline, "cpu_baseline": cpu}
    print(json.dumps(out))


def ptg_clone(ptg, p, tensors):
    q = ptg.MPS(p.qsite, p.qbonds, fill="postpone")
    q.a = [x.copy() for x in tensors]
    return q


def batch_reference_arm(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from pytenet_gb300 import batch
    hs, psis, _ = batch.ising_batch(a.batch_count, a.batch_seed)
    rates = []
    for _ in range(a.steps):
        rate, bsec, sample = batch_cpu_sample(a, hs, psis, a.cpu_instances)
        rates.append(rate)
    value = float(np.mean(rates))
    site_updates = sum(2 * len(h.a) - 1 for h in hs)
    out = {"metric": BATCH_METRIC, "value": value, "unit": "site-updates/s", "n_gpus": a.gpus,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": site_updates / value * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": batch_desc(a)},
           "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": os.cpu_count(),
                            "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------------ precision workload
PREC_METRIC = "TDVP site-updates/s, XXZ L=32 D=1024, mixed vs FP64 per step; DMRG D=1024"


def precision_arm(a):
    """XXZ L=32 (J=1, Delta=0.8, h=-0.1), bonds min(2^min(i, L-i), 1024), seeded random
    left-orthonormal MPS; TDVP dt=0.02j, numiter_lanczos=12 in the mixed form (timed over
    --steps steps) with energy error, norm drift and infidelity against the FP64 form after
    each of the first --acc-steps steps; then single-site DMRG (--dmrg-sweeps sweeps, mixed)
    from a seeded random D=1024 state with the FP64 sweeps' energies for the first
    --dmrg-acc-sweeps sweeps."""
    import torch
    import warnings
    import __graft_entry__
    __graft_entry__.build()
    import pytenet_gb300 as ptg
    from pytenet_gb300 import _lib
    _lib.load()
    L, D, m, dt = 32, 1024, 12, 0.02j
    rng = np.random.default_rng(a.seed)
    h = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    h.zero_qnumbers()
    b = [min(2 ** min(i, L - i), D) for i in range(L + 1)]
    psi = ptg.MPS(h.qsite, [bi * [0] for bi in b], fill="random", rng=rng)
    psi.orthonormalize(mode="left")
    host0 = [x.copy() for x in psi.a]

    def fresh():
        p = ptg.MPS(psi.qsite, psi.qbonds, fill="postpone")
        p.a = [x.copy() for x in host0]
        return p

    # ---- TDVP, mixed, timed; accuracy steps in lockstep with the FP64 form
    pm, pf = fresh(), fresh()
    rm = ptg.TDVPRun(h, pm, numiter_lanczos=m, precision="mixed")
    rf = ptg.TDVPRun(h, pf, numiter_lanczos=m, precision="fp64") if a.acc_steps > 0 else None
    per_step = []
    t_acc = 0.0
    for k in range(a.acc_steps):
        rm.step(dt)
        rf.step(dt)
        # contracted on the device from the runs' resident tensors (no download)
        em, ef = rm.energy().real, rf.energy().real
        ov = rm.vdot(rf)
        nm, nf = rm.vdot(rm).real, rf.vdot(rf).real
        per_step.append({"step": k + 1, "energy_fp64": ef, "energy_mixed": em,
                         "energy_rel_err": abs(em - ef) / abs(ef),
                         "infidelity": 1.0 - abs(ov) ** 2 / (nm * nf),
                         "norm_drift": abs(np.sqrt(nm) - np.sqrt(nf))})
    del rf
    warm = max(0, 3 - a.acc_steps)   # at least 3 untimed steps in all
    for _ in range(warm):
        rm.step(dt)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0.record()
    for _ in range(a.steps):
        rm.step(dt)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    value = (2 * L - 1) * a.steps / (ms / 1e3)
    # ---- DMRG from a seeded random D=1024 state
    rng2 = np.random.default_rng(a.seed + 1)
    hd = ptg.heisenberg_xxz_1d_mpo(L, 1.0, 0.8, -0.1)
    hd.zero_qnumbers()
    p0 = ptg.MPS(hd.qsite, [bi * [0] for bi in b], fill="random", rng=rng2)
    d0 = [x.copy() for x in p0.a]
    pdm = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
    pdm.a = [x.copy() for x in d0]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        t0 = time.perf_counter()
        en_m = ptg.dmrg_singlesite(hd, pdm, a.dmrg_sweeps, numiter_lanczos=m, precision="mixed")
        torch.cuda.synchronize()
        t_dm = time.perf_counter() - t0
        en_f = []
        if a.dmrg_acc_sweeps > 0:
            pdf = ptg.MPS(p0.qsite, p0.qbonds, fill="postpone")
            pdf.a = [x.copy() for x in d0]
            en_f = list(ptg.dmrg_singlesite(hd, pdf, a.dmrg_acc_sweeps, numiter_lanczos=m,
                                            precision="fp64"))
    dmrg = {"sweeps": a.dmrg_sweeps, "numiter_lanczos": m, "energies_mixed": list(map(float, en_m)),
            "energies_fp64": list(map(float, en_f)),
            "energy_rel_err_per_sweep": [abs(float(en_m[k]) - en_f[k]) / abs(en_f[k])
                                         for k in range(len(en_f))],
            "site_updates_per_s": 2 * (L - 1) * a.dmrg_sweeps / t_dm, "seconds": t_dm}
    out = {"metric": PREC_METRIC, "value": value, "unit": "site-updates/s", "n_gpus": 1,
           "steps": a.steps, "warmup": a.acc_steps + warm, "ms_per_step": ms / a.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16 digits (5 x 8-bit fixed point, tcgen05) + f64", "data": "synthetic",
           "config": {"workload": f"XXZ L={L} D={D} J=1 Delta=0.8 h=-0.1 (seed {a.seed}), "
                                  f"dt=0.02j, numiter_lanczos={m}; TDVP steps timed after "
                                  f"{a.acc_steps} accuracy steps",
                      "l2": "inputs larger than L2"},
           "clocks": clk, "accuracy_per_step": per_step, "dmrg": dmrg}
    print(json.dumps(out))


def accuracy_vs_fp64(a, ptg, h, psi_host0, qb0, depth_model=None):
    """The benchmarked form (mixed, with the learned depth when given) and the plain
    FP64 fixed-depth form from the same initial state, stepped in lockstep for
    --acc-steps steps: after every step the energy error, infidelity and norm
    drift against the FP64 form, contracted on the device from the runs' resident
    tensors. The FP64 steps after the first (which captures the CUDA graph) are
    timed with CUDA events: the FP64 GPU form's site-updates/s on the same chain,
    the denominator of the metric's "mixed+learned vs FP64" ratio."""
    import torch
    runs = {}
    for form in ("mixed", "fp64"):
        p = ptg.MPS(h.qsite, qb0, fill="postpone")
        p.a = [x.copy() for x in psi_host0]
        runs[form] = ptg.TDVPRun(h, p, numiter_lanczos=a.m, precision=form, graph=a.graph,
                                 depth_model=depth_model if form == "mixed" else None,
                                 depth_tol=a.depth_tol)
    rm, rf = runs["mixed"], runs["fp64"]
    per_step, fp64_ms = [], []
    for k in range(a.acc_steps):
        rm.step(0.05j)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rf.step(0.05j)
        e1.record()
        torch.cuda.synchronize()
        if k > 0:
            fp64_ms.append(e0.elapsed_time(e1))
        em, ef = rm.energy().real, rf.energy().real
        ov = rm.vdot(rf)
        nm2, nf2 = rm.vdot(rm).real, rf.vdot(rf).real
        per_step.append({"step": k + 1, "energy_fp64": ef, "energy_mixed": em,
                         "energy_rel_err": abs(em - ef) / max(abs(ef), 1e-300),
                         "infidelity": 1.0 - abs(ov) ** 2 / (nm2 * nf2),
                         "norm_drift": abs(np.sqrt(nm2) - np.sqrt(nf2))})
    last = per_step[-1]
    out = {"steps": a.acc_steps, "against": "fp64, fixed depth", "energy_fp64": last["energy_fp64"],
           "energy_mixed": last["energy_mixed"], "energy_rel_err": last["energy_rel_err"],
           "infidelity": last["infidelity"], "norm_drift": last["norm_drift"],
           "worst_energy_rel_err": max(r["energy_rel_err"] for r in per_step),
           "worst_infidelity": max(r["infidelity"] for r in per_step),
           "worst_norm_drift": max(r["norm_drift"] for r in per_step),
           "per_step": per_step}
    fp64 = None
    if fp64_ms:
        ms = float(np.mean(fp64_ms))
        fp64 = {"value": (2 * a.L - 1) / (ms / 1e3), "unit": "site-updates/s",
                "ms_per_step": ms, "steps_timed": len(fp64_ms), "warmup": 1,
                "graph": a.graph,
                "what": "plain complex128 form (FP64 DMMA contractions, FP64 Krylov and QR, "
                        "fixed depth numiter_lanczos) on the same chain and initial state; the "
                        "first step (graph capture) untimed"}
    return out, fp64


# ------------------------------------------------------------------ QR workload

def qr_arm(a):
    """ptn_qr with Q formed on the bulk site-tensor shapes (2D x D), one JSON line:
    median CUDA-event time of 10 calls after 3 warm-up calls, per kernel form
    (block update PTN_TUNE_LARFB_TILE, panel PTN_TUNE_QR_PANEL), and the largest
    elementwise difference of Q and R from numpy.linalg.qr."""
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import ptr, stream_ptr
    L = _lib.load()
    forms = [("earlier three-pass update, one warp per row group", 5, 1),
             ("register-tiled update, warp-0 scalars and gather", 0, 2),
             ("register-tiled update, two warps per row group, reduce-scatter", 0, 3),
             ("register-tiled update, two warps per row group, shared-memory sums (default)", 0, 0)]
    shapes = [(512, 256), (1024, 512), (2048, 1024)]
    if a.qr_default_only:
        forms, shapes = forms[-1:], [(1024, 512)]
    old = (L.ptn_tune_get(_lib.TUNE_LARFB_TILE), L.ptn_tune_get(_lib.TUNE_QR_PANEL))
    res = []
    try:
        for (m, n) in shapes:
            rng = np.random.default_rng(m + n)
            x = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))) / np.sqrt(2)
            q_ref, r_ref = np.linalg.qr(x, mode="reduced")
            k = min(m, n)
            dx = torch.from_numpy(x).cuda()
            work = torch.empty_like(dx)
            q = torch.empty((m, k), dtype=torch.complex128, device="cuda")
            r = torch.empty((k, n), dtype=torch.complex128, device="cuda")
            for what, lt, pn in forms:
                _lib.check(L.ptn_tune_set(_lib.TUNE_LARFB_TILE, lt))
                _lib.check(L.ptn_tune_set(_lib.TUNE_QR_PANEL, pn))
                wsb = L.ptn_qr_workspace_bytes(m, n)
                ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
                times = []
                for it in range(13):
                    work.copy_(dx)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    _lib.check(L.ptn_qr(ptr(work), m, n, ptr(q), k, ptr(r), n, ptr(ws), wsb,
                                        stream_ptr()))
                    e1.record()
                    torch.cuda.synchronize()
                    if it >= 3:
                        times.append(e0.elapsed_time(e1))
                ms = float(np.median(times))
                flops = 2 * 8.0 * (m * n * k - (m + n) * k * k / 2.0 + k ** 3 / 3.0)
                res.append({"m": m, "n": n, "form": what, "larfb_tile": lt, "qr_panel": pn,
                            "ms": ms, "fp64_tflops": flops / (ms * 1e-3) / 1e12,
                            "max_err_q": float(np.abs(q.cpu().numpy() - q_ref).max()),
                            "max_err_r": float(np.abs(r.cpu().numpy() - r_ref).max())})
    finally:
        L.ptn_tune_set(_lib.TUNE_LARFB_TILE, old[0])
        L.ptn_tune_set(_lib.TUNE_QR_PANEL, old[1])
    best = min(x["ms"] for x in res if (x["m"], x["n"]) == (1024, 512))
    print(json.dumps({"metric": "ptn_qr time, complex128 1024x512 with Q formed", "value": best,
                      "unit": "ms", "higher_is_better": False, "dtype": "c128",
                      "data": "synthetic",
                      "config": {"workload": "ptn_qr (Q and R) of seeded complex Gaussian "
                                             "matrices, median of 10 timed calls"},
                      "forms": res}))


def main():
    a = parse()
    if a.workload == "qr":
        qr_arm(a)
        return
    if a.workload == "xxz-d1024":
        precision_arm(a)
        return
    if a.workload == "ising-batch":
        if a.impl == "reference":
            batch_reference_arm(a)
        else:
            batch_arm(a)
    elif a.impl == "reference":
        reference_arm(a)
    else:
        our_arm(a)


if __name__ == "__main__":
    main()
