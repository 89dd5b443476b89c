"""Benchmark: MPO.MPS + TT-SVD-round sweeps/s at chi=256 (config 2).

Workload (one "step" = one sweep): a random MPS with N=64 sites, d=2, uniform
bond chi=256 (entries N(0,1)/sqrt(chi*d)) and a random MPO with N=64, d=2x2,
bond D=16 (entries N(0,1)/sqrt(D*d)), both seeded and synthetic.  A sweep is
the raw product W @ X (bond chi*D = 4096), its TT-SVD rounding back to chi=256
and the overlap <X|Z> of the rounded state with the input.

  value       sweeps/s of the chosen form (default: BF16X6, FP64-class on the
              bf16 tensor cores) with the cores already resident in HBM
  e2e         the same through the public API ((W @ X) >> chi, X | Z) with the
              input cores copied from pinned host memory every step and <X|Z>
              read back
  latency     p50/p99 per job (one job = one sweep), on the device and through
              the API
  plain_fp64  sweeps/s of the plain FP64 GPU form (Householder QR + FP64
              Jacobi), the denominator of the metric, and the error of the
              chosen form against it
  roofline    the sliced tensor-core GEMM against the measured bf16 peak,
              timed with CUDA events over the timed region
  phases_ms   one extra sweep split by the rounding's phases (CUDA events)
  cpu_baseline the numpy FP64 port of the same sweep on the host cores: one
              whole measured sweep, plus a 1-thread figure

`--impl reference` times that CPU port alone (the reference itself is pure
Python/numpy and has no GPU path; its own MPS/MPO code cannot run this
workload, see the design notes).  Under torchrun every rank runs an
independent replica (the single-chain sweep does not shard).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SITES, D_PHYS, CHI, D_MPO = 64, 2, 256, 16
SEED = 2024
METRIC = "MPO·MPS+SVD-round sweeps/s at χ=256 vs plain FP64 GPU; p50/p99 job latency"
# precision form -> library code (include/syngular_gb300.h SGT_PREC_*) and the arithmetic it computes in
PRECISIONS = {"f64": 0, "tf32": 1, "tf32x3": 4, "bf16x6": 5}
DTYPES = {"f64": "f64", "tf32": "tf32/f32", "tf32x3": "tf32x3/f32",
          "bf16x6": "bf16x6 slices (tcgen05) / f32 pairs / purification (spectra: f32 Jacobi + refinement)"}


def _eig_profile(enable):
    """Start (True) or stop (False) the eigensolver's event timing.  Stop
    returns (ms, flops, launches); a failure returns its message instead, so
    the measurement never costs the benchmark line."""
    import ctypes

    try:
        from syngular_gb300 import _lib as L

        if enable:
            L.call("sgt_eig_profile", 1, None, None, None)
            return True
        ms, fl, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        L.call("sgt_eig_profile", 0, ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(n))
        return (ms.value, fl.value, n.value)
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return "%s: %s" % (type(e).__name__, e)


def _eig_summary(stats, ms_total, kernel="gjacobi_kernel<1>"):
    """dominant_kernel object: gjacobi_kernel<1>'s mean CUDA-event launch time
    over the timed region, its share of the step, and its FP32 rate (sweeps x
    n(n-1)/2 pair visits x 12 n flops per launch) against the nominal FP32
    CUDA-core rate (152 SMs x 128 lanes x 2 flops x max SM clock; the measured
    peaks hold no FP32 figure) and against the 16 SMs of its one cluster."""
    if not isinstance(stats, tuple):
        return {"kernel": kernel, "error": str(stats)}
    ms, fl, n = stats
    if n <= 0 or ms <= 0:
        return {"kernel": kernel, "launches": int(n)}
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f).get("sm_max_mhz") or mhz)
    except (OSError, ValueError):
        pass
    peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
    achieved = fl / (ms / 1e3) / 1e12
    return {
        "kernel": kernel, "launches": int(n), "ms_per_launch": ms / n,
        "share_of_step": ms / ms_total if ms_total > 0 else None,
        "bound": "latency: one 16-CTA cluster, shared-memory resident, sequential block steps",
        "achieved": achieved, "unit": "TFLOP/s (FP32)", "peak": peak,
        "peak_note": "nominal FP32 CUDA-core rate of all 152 SMs at the max SM clock",
        "frac": achieved / peak, "frac_of_cluster_sms": achieved / (peak * 16 / 152),
    }


def _apply_split(args, L):
    """--split CTAS,KTILES sets the sliced GEMM's split-K shape (library
    tuning); returns the shape in effect."""
    if args.split:
        ctas, kt = (int(v) for v in args.split.split(","))
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_CTAS, ctas)
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_MIN_KTILES, kt)
    if args.pchol:
        L.call("sgt_set_tuning", L.TUNE_PCHOL_BLOCKED, {"cluster": 0, "blocked": 1}[args.pchol])
    if args.purify_step:
        L.call("sgt_set_tuning", L.TUNE_PURIFY_VECTOR_STEP, {"warp": 0, "block": 1}[args.purify_step])
    lib = L.load()
    return {"split_ctas": int(lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS)),
            "split_min_ktiles": int(lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES)),
            "pivoted_cholesky": "blocked" if lib.sgt_get_tuning(L.TUNE_PCHOL_BLOCKED) else "cluster",
            "purify_step": "block" if lib.sgt_get_tuning(L.TUNE_PURIFY_VECTOR_STEP) else "warp"}


def _pct(values, p):
    """Nearest-rank percentile of a small sample (None when empty)."""
    v = sorted(values)
    if not v:
        return None
    return v[min(len(v) - 1, max(0, int(math.ceil(p / 100.0 * len(v))) - 1))]


def workload_name():
    return ("config2: MPS N=%d d=2 chi=256 x MPO D=16 -> raw product (bond 4096) -> TT-SVD round to chi=256 -> <X|Z>"
            % N_SITES) + ("" if N_SITES == 64 else " (shortened chain for profiling, not the headline)")


def make_inputs():
    """Seeded config-2 cores (numpy float64)."""
    import numpy as np

    rng = np.random.default_rng(SEED)
    dims = [1] + [CHI] * (N_SITES - 1) + [1]
    X = [rng.standard_normal((dims[k], D_PHYS, dims[k + 1])) / math.sqrt(max(dims[k], dims[k + 1]) * D_PHYS)
         for k in range(N_SITES)]
    wd = [1] + [D_MPO] * (N_SITES - 1) + [1]
    W = [rng.standard_normal((wd[k], D_PHYS, D_PHYS, wd[k + 1])) / math.sqrt(max(wd[k], wd[k + 1]) * D_PHYS)
         for k in range(N_SITES)]
    return X, W


# ---------------------------------------------------------------------------
# clocks sampling
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU port (the oracle) on a bounded sample
# ---------------------------------------------------------------------------

def site_flops_model():
    """Per-site flops of the TT-SVD sweep at config 2 (left QR step and right
    SVD step), by site shape; returns (list, index of a middle site)."""
    b = [1]
    R = [1] + [CHI * D_MPO] * (N_SITES - 1) + [1]
    for k in range(N_SITES - 1):
        b.append(min(b[k] * D_PHYS, R[k + 1]))
    x = [1] * (N_SITES + 1)
    for k in range(N_SITES - 1, 0, -1):
        x[k] = min(CHI, b[k], D_PHYS * x[k + 1])
    fl = []
    for k in range(N_SITES):
        m, n = b[k] * D_PHYS, R[k + 1]
        q = min(m, n)
        left = 2 * m * n * q - 2 * q ** 3 / 3 + 2 * q * R[k + 1] * D_PHYS * R[min(k + 2, N_SITES)] if k < N_SITES - 1 else 0
        c = D_PHYS * x[k + 1]
        mm = b[k]
        right = 2 * mm * c * min(mm, c) + 10 * min(mm, c) ** 3 + 2 * (b[k - 1] * D_PHYS if k else 1) * mm * x[k] if k else 0
        fl.append(left + right)
    mid = N_SITES // 2
    return fl, mid


def cpu_site_sample(rng_seed=7):
    """One full-size middle site of the numpy FP64 sweep: left QR step
    (reduced QR of the 8192 x 4096 carried core + the carry GEMM into the next
    product core) and right SVD step (QR of 4096 x 512, SVD of 512 x 512,
    push of U*S through Q).  Returns seconds."""
    import numpy as np

    from oracle import tt_fp64 as O

    rng = np.random.default_rng(rng_seed)
    R = CHI * D_MPO
    x = O.random_mps_cores(rng, 3, D_PHYS, CHI)
    w = O.random_mpo_cores(rng, 3, D_PHYS, D_MPO)
    P = O.mpo_mps_product(w[1:2], x[1:2])[0]  # (4096, 2, 4096)
    Pn = O.mpo_mps_product(w[1:2], x[1:2])[0]
    t0 = time.perf_counter()
    C = P.reshape(R * D_PHYS, R)
    Q, Rf = np.linalg.qr(C)
    Cn = Rf @ Pn.reshape(R, -1)
    M = Cn.reshape(R, -1)[:, : D_PHYS * CHI]
    Qm, Rm = np.linalg.qr(M)
    U, s, Vt = np.linalg.svd(Rm)
    US = (Qm @ U[:, :CHI]) * s[:CHI]
    pushed = Q @ US
    t1 = time.perf_counter()
    del pushed
    return t1 - t0


def cpu_info():
    """CPU model, core count and the BLAS build numpy uses (printed with every
    CPU figure)."""
    import numpy as np

    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                key = ln.split(":")[0].strip().lower()
                if key in ("model name", "cpu part", "hardware") and model is None:
                    model = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    blas = None
    try:
        b = np.show_config(mode="dicts")["Build Dependencies"]["blas"]
        blas = "%s %s (%s)" % (b.get("name"), b.get("version"), b.get("openblas configuration", ""))
    except Exception:  # noqa: BLE001 - informational only
        pass
    return {"cpu_model": model, "cores": os.cpu_count(), "blas": blas, "numpy": np.__version__}


_CPU_SWEEP = """
import json, sys, time
sys.path.insert(0, %r)
import bench
bench.N_SITES = %d
from oracle import tt_fp64 as O
X, W = bench.make_inputs()
t0 = time.perf_counter()
Z, ov, spectra, disc = O.sweep_fp64(W, X, bench.CHI)
print(json.dumps({"seconds": time.perf_counter() - t0, "overlap": ov}))
"""

_CPU_SITE = """
import json, sys
sys.path.insert(0, %r)
import bench
print(json.dumps({"seconds": bench.cpu_site_sample()}))
"""


def _cpu_subprocess(code, threads):
    """Run a CPU measurement in a fresh interpreter whose BLAS uses `threads`
    threads (the thread count is fixed when numpy loads its BLAS)."""
    env = dict(os.environ)
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        env[var] = str(threads)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("CPU measurement failed: %s" % r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_full_sweep(threads, sites=None):
    """One whole sweep of the numpy FP64 port (the oracle: raw product, left QR
    sweep, right-to-left SVDs, overlap) on the host cores; returns seconds."""
    return _cpu_subprocess(_CPU_SWEEP % (ROOT, sites or N_SITES), threads)


def cpu_baseline_measure():
    """The numpy FP64 port on the host cores: one measured full sweep with all
    cores, plus a 1-thread figure (one full-size middle site at one thread,
    scaled to the sweep by per-site flops: a full 1-thread sweep takes ~40 min)."""
    cores = os.cpu_count() or 1
    full = cpu_full_sweep(cores)
    t_sweep = full["seconds"]
    fl, mid = site_flops_model()
    scale = sum(fl) / fl[mid]
    one = _cpu_subprocess(_CPU_SITE % ROOT, 1)["seconds"] * scale
    info = cpu_info()
    return {"value": 1.0 / t_sweep, "unit": "sweeps/s", "cores": cores, "kind": "port",
            "sample": "one whole %d-site sweep of the numpy FP64 port (measured, %.1f s, all %d host threads)"
                      % (N_SITES, t_sweep, cores),
            "seconds_per_sweep": t_sweep, "overlap": full["overlap"],
            "one_thread": {"value": 1.0 / one, "unit": "sweeps/s", "cores": 1,
                           "sample": "one full-size middle site at 1 thread, scaled to the sweep by per-site "
                                     "flops (x%.1f)" % scale, "seconds_per_sweep": one},
            **info}


def run_reference(args, rank, world):
    """The reference arm: the numpy FP64 port of the sweep (the reference's own
    MPS / MPO code cannot run this workload), whole sweeps on all host cores.
    A sweep takes minutes, so the arm runs one untimed sweep of a 3-site chain
    of the same core shapes and then exactly one timed full sweep, and reports
    the steps it ran (1)."""
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    cpu_full_sweep(cores, sites=3)  # warm-up (BLAS threads, page-in)
    full = cpu_full_sweep(cores)
    t_sweep = full["seconds"]
    v = 1.0 / t_sweep
    info = cpu_info()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "sweeps/s", "n_gpus": world,
        "steps": 1, "warmup": 1, "ms_per_step": t_sweep * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, config-2 shapes)",
        "config": {"workload": workload_name(), "cpu": "numpy FP64 port of the sweep (Householder QR + LAPACK SVD)",
                   "steps_note": "one whole sweep timed (about %.0f s); the --steps / --warmup values asked "
                                 "for (%d / %d) are not run: each would be a further whole sweep"
                                 % (t_sweep, args.steps, args.warmup)},
        "cpu_baseline": {"value": v, "unit": "sweeps/s", "cores": cores, "kind": "port",
                         "sample": "one whole %d-site sweep (measured), after a 3-site warm-up sweep" % N_SITES,
                         **info},
        "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "overlap": full["overlap"],
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_gpu(args, rank, world, local_rank):
    import ctypes

    import numpy as np
    import torch
    import torch.distributed as dist

    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    prec = PRECISIONS[args.precision]
    split = _apply_split(args, L)

    Xh, Wh = make_inputs()
    Xd = [torch.from_numpy(c).to(dev) for c in Xh]
    Wd = [torch.from_numpy(c).to(dev) for c in Wh]
    Xp = [torch.from_numpy(c).pin_memory() for c in Xh]
    Wp = [torch.from_numpy(c).pin_memory() for c in Wh]
    h2d = sum(c.size * 8 for c in Xh) + sum(c.size * 8 for c in Wh)

    # the metric's operation, as `(W @ X) >> chi` returns it: rounded cores (and
    # discarded weights), no per-bond spectra; `spectra=True` times the variant
    # that also returns every bond's singular values (an eigensolve per bond)
    # the overlap in the same form (BF16X6: contractions on the sliced GEMM)
    oprec = prec if prec == L.PREC_BF16X6 else L.PREC_F64

    def step(X, W, spectra=False):
        Z, spec, counts, disc, status = _ops.mpo_mps_round(W, X, CHI, prec, spectra=spectra)
        res = _ops.overlap_device(X, Z, oprec)
        return Z, res, status

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(v):
        if world > 1:
            t = torch.tensor([v], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return v

    # warm-up
    for _ in range(max(args.warmup, 3)):
        Z, res, status = step(Xd, Wd)
    torch.cuda.synchronize()
    st = int(status.item())
    if st < 0:
        raise RuntimeError("round did not converge (status %d)" % st)

    # ---- timed region: device-resident inputs ----
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    L.call("sgt_tc_profile", 1, None, None, None)
    L.call("sgt_sliced_profile", 1, None, None, None)
    eig_prof = _eig_profile(True)
    launches0 = L.load().sgt_launch_count()
    barrier()
    torch.cuda.synchronize()
    # one event per step boundary: the K steps are also K jobs whose device
    # latencies give the p50/p99 of the metric
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    e0, e1 = evs[0], evs[-1]
    e0.record()
    for i in range(args.steps):
        Z, res, status = step(Xd, Wd)
        evs[i + 1].record()
    torch.cuda.synchronize()
    barrier()
    step_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    launches = L.load().sgt_launch_count() - launches0
    tc_ms, tc_flops, tc_n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
    L.call("sgt_tc_profile", 0, ctypes.byref(tc_ms), ctypes.byref(tc_flops), ctypes.byref(tc_n))
    oz_ms, oz_flops, oz_n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
    L.call("sgt_sliced_profile", 0, ctypes.byref(oz_ms), ctypes.byref(oz_flops), ctypes.byref(oz_n))
    eig_stats = _eig_profile(False) if eig_prof is True else eig_prof
    clk = clocks.stop()
    ms_total = max_over_ranks(e0.elapsed_time(e1))
    ms_step = ms_total / args.steps
    value = world * args.steps / (ms_total / 1e3)
    ov_fast = _ops.decode_overlap(res.cpu().tolist())

    # ---- e2e: host buffers in, scalar out, through the drop-in API ----
    # (W @ X) >> chi with the raw product left unformed (AUTO_ROUND off) and the
    # TT-SVD rounding in the benchmark's precision, then X | Z back on the host
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    saved = (MatrixProductOperator.AUTO_ROUND, MatrixProductOperator.PRECISION, MatrixProductState.ROUNDING,
             MatrixProductState.PRECISION)
    MatrixProductOperator.AUTO_ROUND = False
    MatrixProductOperator.PRECISION = args.precision
    MatrixProductState.ROUNDING = "svd"
    MatrixProductState.PRECISION = args.precision
    try:
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        e2e_job_ms = []
        for _ in range(args.steps):
            tj = time.perf_counter()
            Xm = MatrixProductState.from_sites([c.to(dev, non_blocking=True) for c in Xp])
            Wm = MatrixProductOperator.from_sites([c.to(dev, non_blocking=True) for c in Wp])
            Zm = (Wm @ Xm) >> CHI
            ov_api = float(Xm | Zm)
            e2e_job_ms.append((time.perf_counter() - tj) * 1e3)
        torch.cuda.synchronize()
        barrier()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
    finally:
        (MatrixProductOperator.AUTO_ROUND, MatrixProductOperator.PRECISION, MatrixProductState.ROUNDING,
         MatrixProductState.PRECISION) = saved
    e2e_value = world * args.steps / e2e_s

    out = {
        "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded N(0,1)/sqrt(chi*d) cores)",
        "config": {"workload": workload_name(), "form": args.precision, "tuning": split, "l2": "working set larger than L2 every step (bf16x6: %.1f GB of Gram-matrix slices written and "
                   "read per sweep; tf32 forms: %.1f GB of split product cores)"
                   % (N_SITES * 4096 * 4096 * 12 / 1e9, N_SITES * 4096 * 2 * 4096 * 8 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "sweeps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 16,
                "api": "(MatrixProductOperator @ MatrixProductState) >> chi with AUTO_ROUND=False, ROUNDING='svd', "
                       "PRECISION='%s' on both classes; then X | Z" % args.precision, "overlap": ov_api},
        "latency": {"p50_ms": _pct(step_ms, 50), "p99_ms": _pct(step_ms, 99), "jobs": len(step_ms),
                    "e2e_p50_ms": _pct(e2e_job_ms, 50), "e2e_p99_ms": _pct(e2e_job_ms, 99),
                    "note": "one job = one sweep; device time per step (inputs resident) and wall time per "
                            "API call with host inputs and the overlap read back"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "overlap": ov_fast,
        "jacobi_sweeps_max": int(status.item()),
    }
    # the dominant kernel (the bond eigensolver), from its live events
    # the form's first-approximation method: 2 for bf16x6 unless SGT_EIG_METHOD chooses
    meth = int(os.environ.get("SGT_EIG_METHOD", "0") or 0)
    if meth not in (1, 2, 3):
        meth = 2 if args.precision == "bf16x6" else 1
    out["eigensolver"] = _eig_summary(eig_stats, ms_total, "gjacobi_kernel<%d>" % meth)
    # roofline of the contractions (tcgen05 GEMM), from the live events
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("bf16_tflops") or 1900.0
    passes = 3 if args.precision == "tf32x3" else 1
    if oz_n.value > 0:
        # sliced bf16 GEMM: 21 slice-pair MMAs of 2MNK each per FP64-class product
        per_launch_s = oz_ms.value / 1e3 / oz_n.value
        alg_flops = oz_flops.value / oz_n.value
        achieved = alg_flops * 21 / per_launch_s / 1e12
        out["roofline"] = {
            "bound": "tensor", "kernel": "oz_gemm_kernel", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
            "note": "bf16 tensor-pipe flops (21 slice products x 2MNK) per launch / mean CUDA-event launch time "
                    "over the timed region (split-K reduction included); peak = measured dense bf16 (burst)",
            "share_of_step": oz_ms.value / ms_total if ms_total > 0 else None,
            "launches": oz_n.value, "fp64_equivalent_tflops": alg_flops / per_launch_s / 1e12,
        }
    if tc_n.value > 0:
        per_launch_s = tc_ms.value / 1e3 / tc_n.value
        alg_flops = tc_flops.value / tc_n.value
        achieved = alg_flops * passes / per_launch_s / 1e12
        traffic = None
        # DRAM bytes per launch of this kernel over the sweep's launch mix, from
        # an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum)
        tpath = os.path.join(ROOT, "profiles", "tc_gemm_tf32_traffic.txt")
        if os.path.exists(tpath):
            with open(tpath) as f:
                for ln in f:
                    if ln.startswith("bytes_per_launch"):
                        traffic = float(ln.split()[1])
        out["roofline"] = {
            "bound": "tensor", "kernel": "tc_gemm_tf32_kernel", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
            "note": "tensor-pipe TF32 flops (%d pass(es) x 2MNK) per launch / mean CUDA-event launch time over "
                    "the timed region; peak = measured dense bf16 (TF32 issues at half that rate)" % passes,
            "share_of_step": tc_ms.value / (ms_total * 1.0) if ms_total > 0 else None,
            "launches": tc_n.value,
        }
    # the kernel with the largest share of the step
    shares = {}
    if isinstance(out.get("eigensolver"), dict) and out["eigensolver"].get("share_of_step"):
        shares["eigensolver"] = out["eigensolver"]["share_of_step"]
    if "roofline" in out and out["roofline"].get("share_of_step"):
        shares["roofline"] = out["roofline"]["share_of_step"]
    if shares:
        top = max(shares, key=shares.get)
        out["dominant_kernel"] = dict(out[top])
    # where one sweep's time goes (an extra, untimed sweep with CUDA events at
    # the rounding's phase boundaries)
    if prec == L.PREC_BF16X6:
        try:
            names = ["left_gram", "projections_Y", "bond_matrices_Z", "purification", "kept_basis",
                     "discarded", "carry_F", "eigensolve"]
            buf = (ctypes.c_double * len(names))()
            torch.cuda.synchronize()
            L.call("sgt_phase_profile", 1, None, 0)
            q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            q0.record()
            Z, res, status = step(Xd, Wd)
            q1.record()
            torch.cuda.synchronize()
            L.call("sgt_phase_profile", 0, buf, len(names))
            out["phases_ms"] = {nm: buf[i] for i, nm in enumerate(names)}
            out["phases_ms"]["sweep_total"] = q0.elapsed_time(q1)
        except Exception as e:  # noqa: BLE001 - reported in the JSON line
            out["phases_ms"] = {"error": "%s: %s" % (type(e).__name__, e)}
    # the variant with every bond's spectrum (eigensolve per bond), same inputs
    if prec == L.PREC_BF16X6 and not args.no_spectra_variant:
        step(Xd, Wd, spectra=True)
        torch.cuda.synchronize()
        v0, v1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ns = max(1, min(args.steps, 3))
        v0.record()
        for _ in range(ns):
            Zs_, res_s, st_s = step(Xd, Wd, spectra=True)
        v1.record()
        torch.cuda.synchronize()
        ms_s = max_over_ranks(v0.elapsed_time(v1)) / ns
        out["with_spectra"] = {"sweeps_per_s": world * 1e3 / ms_s, "ms_per_sweep": ms_s, "steps": ns,
                               "overlap": _ops.decode_overlap(res_s.cpu().tolist()),
                               "note": "the same sweep also returning every bond's singular values: FP32 Jacobi "
                                       "+ refinement per bond instead of the purification"}
    # plain FP64 GPU form (denominator) and the error of the fast form against it
    if not args.no_plain and prec != L.PREC_F64:
        torch.cuda.synchronize()
        # warm the FP64 kernels on a short chain with the same core shapes
        Xs = [Xd[0], Xd[1], Xd[-1]]
        Ws = [Wd[0], Wd[1], Wd[-1]]
        _ops.mpo_mps_round(Ws, Xs, CHI, L.PREC_F64)
        torch.cuda.synchronize()
        plain_runs = []
        for _ in range(max(1, args.plain_steps)):
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record()
            Zp, spec_p, counts_p, disc_p, status_p = _ops.mpo_mps_round(Wd, Xd, CHI, L.PREC_F64)
            resp = _ops.overlap_device(Xd, Zp)
            p1.record()
            torch.cuda.synchronize()
            plain_runs.append(max_over_ranks(p0.elapsed_time(p1)))
        plain_ms = statistics.mean(plain_runs)
        ov_plain = _ops.decode_overlap(resp.cpu().tolist())
        nx = math.sqrt(_ops.overlap(Xd, Xd))
        nz = math.sqrt(abs(_ops.overlap(Zp, Zp)))
        out["plain_fp64"] = {"sweeps_per_s": world * 1e3 / plain_ms, "ms_per_sweep": plain_ms,
                             "steps": len(plain_runs), "ms_each": plain_runs,
                             "spread_rel": (max(plain_runs) - min(plain_runs)) / plain_ms,
                             "warmup": "one 3-site chain of the same core shapes", "status": int(status_p.item())}
        out["speedup_vs_plain_fp64"] = value / (world * 1e3 / plain_ms)
        # 1 - |<Z|Z_fp64>| / (|Z| |Z_fp64|): how far the rounded state of the
        # fast form is from the FP64 one (gauge-invariant)
        nzf = math.sqrt(abs(_ops.overlap(Z, Z)))
        fid = abs(_ops.overlap(Z, Zp)) / (nzf * nz)
        out["error_vs_fp64"] = {"overlap_rel": abs(ov_fast - ov_plain) / abs(ov_plain),
                                "overlap_norm": abs(ov_fast - ov_plain) / (nx * nz),
                                "overlap_fp64": ov_plain, "state_infidelity": 1.0 - fid,
                                "norm_rel": abs(nzf - nz) / nz}
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_measure()
    if rank == 0:
        print(json.dumps(out))
    return 0


# ---------------------------------------------------------------------------
# secondary workloads: batched uneven instances, serving stream
# ---------------------------------------------------------------------------

def config3_instances(count=512, seed=3):
    """Batched workload: count independent pairs, N ~ U[8,64], d in {2,3,4},
    chi ~ U[16,128], D in {4,8,16}, entries N(0,1)/sqrt(chi*d)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(8, 65))
        d = int(rng.choice([2, 3, 4]))
        chi = int(rng.integers(16, 129))
        D = int(rng.choice([4, 8, 16]))
        dims = [1] + [chi] * (n - 1) + [1]
        X = [rng.standard_normal((dims[k], d, dims[k + 1])) / math.sqrt(chi * d) for k in range(n)]
        wd = [1] + [D] * (n - 1) + [1]
        W = [rng.standard_normal((wd[k], d, d, wd[k + 1])) / math.sqrt(D * d) for k in range(n)]
        out.append((W, X, chi))
    return out


def run_batched(args):
    """Config 3: independent instances through one batched plan per GPU,
    replayed as a captured CUDA graph.  Under torchrun the instances are dealt
    across ranks (shard: no data exchange, every instance is independent); each
    rank times its own share between barriers and the line reports all
    instances over the slowest rank's time."""
    import torch
    import torch.distributed as dist

    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.batched import BatchedRound, Instance, autotune, shard

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    def reduce(v, op):
        if world == 1:
            return v
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=op)
        return float(t.item())

    t_start = time.perf_counter()

    def log(msg):
        if rank == 0:
            print("[batched %7.1f s] %s" % (time.perf_counter() - t_start, msg), file=sys.stderr, flush=True)

    prec = PRECISIONS[args.precision]
    data = config3_instances(args.instances)
    mine = shard(list(range(len(data))), rank, world)
    insts = [Instance(*data[i]) for i in mine]
    log("%d instances, %d on this rank" % (len(data), len(insts)))
    # the batch returns rounded cores and overlaps (no per-bond spectra)
    # lane count timed on a sample of the batch (graph replays), then used for all of it
    tune = autotune(insts[: min(len(insts), 128)], precision=prec, candidates=(4, 8, 16), reps=1, spectra=False,
                    per_lane=args.graph_per_lane,
                    splits=((148, 8), (152, 4), (304, 4)) if prec == L.PREC_BF16X6 else ())
    log("autotune: %s" % json.dumps(tune))
    b = BatchedRound(insts, precision=prec, streams=tune["streams"], spectra=False)
    b.capture(per_lane=args.graph_per_lane)
    log("%d graph(s) captured" % len(b.graphs))
    for _ in range(max(args.warmup, 3)):
        b.replay()
    torch.cuda.synchronize()
    log("warm-up replays done")
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        b.replay()
    e1.record()
    torch.cuda.synchronize()
    barrier()
    ms = reduce(e0.elapsed_time(e1) / args.steps, dist.ReduceOp.MAX if world > 1 else None)
    st = b.statuses()
    converged = int(reduce(sum(1 for x in st if x >= 0), dist.ReduceOp.SUM if world > 1 else None))
    log("timed replays: %.1f ms per batch" % ms)
    # plain FP64 per-instance form on a sample, scaled to the batch by instance count;
    # the fast form's overlaps are read first (the FP64 plan re-binds the
    # instances' output buffers)
    sample = insts[: args.plain_sample]
    fast_ovl = b.overlaps()[: len(sample)]
    bp = BatchedRound(sample, precision=L.PREC_F64, streams=1, spectra=False)
    bp.launch()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record()
    bp.launch()
    p1.record()
    torch.cuda.synchronize()
    plain_ms_per_inst = p0.elapsed_time(p1) / len(sample)
    # error of the batched form against the plain FP64 form on the sample
    from syngular_gb300.tensor._ops import decode_overlap

    errs = []
    for a, plain in zip(fast_ovl, bp.instances):
        r = decode_overlap(plain.ovl.cpu().tolist())
        errs.append(abs(a - r) / abs(r) if r != 0 else abs(a))
    log("plain FP64 sample: %.1f ms per instance" % plain_ms_per_inst)
    out = {
        "metric": "batched MPO.MPS+TT-SVD-round+overlap instances/s", "value": len(data) / (ms / 1e3),
        "unit": "instances/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms, "higher_is_better": True, "scaling": "strong" if world > 1 else "weak",
        "dtype": DTYPES[args.precision], "data": "synthetic (seeded)",
        "config": {"workload": "config3: %d instances, N~U[8,64], d in {2,3,4}, chi~U[16,128], D in {4,8,16}"
                   % len(data), "streams": tune["streams"],
                   "graph": "%d captured CUDA graph(s) per batch and rank, replayed back to back" % len(b.graphs),
                   "autotune": tune, "parallelism": "instances sharded over %d rank(s)" % world},
        "converged": converged, "instances": len(data), "plain_fp64_instances_per_s": 1e3 / plain_ms_per_inst,
        "plain_fp64_sample": len(sample),
        "overlap_error_vs_fp64_on_sample": {"max_rel": max(errs), "median_rel": statistics.median(errs)},
    }
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()
    return 0


def config4_inputs(n=32, d=2, chi=1024, ratio=0.98, seed=4):
    """Two MPS with geometric bond spectra s_k ~ ratio**k: every core is a random
    orthogonal factor x diag(s) x a random orthogonal factor, bonds capped by the
    rank bound at the edges."""
    import numpy as np

    rng = np.random.default_rng(seed)
    dims = [1] + [min(chi, d ** min(k, n - k)) for k in range(1, n)] + [1]

    def chain():
        out = []
        for k in range(n):
            l, r = dims[k], dims[k + 1]
            m = l * d
            q1, _ = np.linalg.qr(rng.standard_normal((m, m)))
            q2, _ = np.linalg.qr(rng.standard_normal((r, r)))
            kk = min(m, r)
            core = (q1[:, :kk] * ratio ** np.arange(kk)) @ q2[:kk, :]
            out.append(core.reshape(l, d, r))
        return out

    return chain(), chain()


def run_config4(args):
    import numpy as np
    import torch

    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    t_start = time.perf_counter()

    def log(msg):
        print("[config4 %7.1f s] %s" % (time.perf_counter() - t_start, msg), file=sys.stderr, flush=True)

    A, B = config4_inputs()
    Ad = [torch.from_numpy(c).cuda() for c in A]
    Bd = [torch.from_numpy(c).cuda() for c in B]
    log("inputs resident")
    S = _ops.concat(Ad, Bd)
    prec = PRECISIONS[args.precision]
    # `>> 1024` returns the rounded state (no per-bond spectra): in BF16X6 the
    # kept subspaces come from the purification, in FP64 from the Jacobi SVDs.
    # The middle bonds here have ~700 directions above the products' noise
    # against 1024 kept, so the purification's clean-up steps are switched on.
    spectra = prec == L.PREC_F64
    if prec == L.PREC_BF16X6:
        L.call("sgt_set_tuning", L.TUNE_PURIFY_CLEANUP, 1)
    for _ in range(args.warmup):
        Z, spec, counts, disc, status = _ops.svd_round(S, 1024, prec, spectra=spectra)
    torch.cuda.synchronize()
    log("warm-up done")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        S = _ops.concat(Ad, Bd)
        Z, spec, counts, disc, status = _ops.svd_round(S, 1024, prec, spectra=spectra)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    log("timed rounds done: %.1f ms each" % ms)
    # Gauge-invariant checks.  The exact rounding discards a weight of ~1e-22
    # of |S|^2 at these spectra (the FP64 oracle's figure), so <S|Z> equals
    # <S|S> and |Z| equals |S| to far below any precision form's error: both
    # are the FP64 answers, without a 334 s FP64 round in the benchmark.
    ss = _ops.overlap(S, S)
    zz = _ops.overlap(Z, Z)
    sz = _ops.overlap(S, Z)
    out = {
        "metric": "config4 round(A + B) to chi=1024 per second", "value": 1e3 / ms, "unit": "rounds/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "dtype": DTYPES[args.precision],
        "data": "synthetic seeded: geometric spectra 0.98^k, random orthogonal factors",
        "config": {"workload": "config4: two MPS N=32 d=2 chi=1024 -> direct sum (bond 2048) -> TT-SVD round "
                               "to 1024", "form": args.precision,
                   "purify_cleanup": int(L.load().sgt_get_tuning(L.TUNE_PURIFY_CLEANUP))},
        "status": int(status.item()),
        "error_vs_fp64": {"overlap_rel": abs(sz - ss) / abs(ss), "norm_rel": abs(math.sqrt(zz) - math.sqrt(ss)) /
                          math.sqrt(ss), "state_infidelity": max(0.0, 1.0 - sz * sz / (ss * zz)),
                          "note": "against the unrounded sum S: the FP64 rounding discards ~1e-22 of |S|^2 here"},
        "discarded_max": float(disc.max().item()),
        "bond_problem": "2048 x 2048 bond matrices at the middle bonds, keep 1024",
    }
    if args.config4_spectra:
        # the variant that also returns every bond's singular values
        Zs_, spec_s, counts_s, disc_s, st_s = _ops.svd_round(S, 1024, prec, spectra=True)
        torch.cuda.synchronize()
        out["with_spectra"] = {"status": int(st_s.item()), "spectra": [float(v) for v in spec_s[:8].cpu()]}
    print(json.dumps(out))
    return 0


def run_hbm(args):
    """The HBM-bound kernels at the benchmark's sizes, each timed with CUDA
    events over --steps launches after --warmup (inputs resident, outputs
    overwritten; every working set is larger than L2 or the per-launch bytes
    are reported as such):
      contract  one product core P (4096, 2, 4096) FP64 = X (256, 2, 256) x W (16, 2, 2, 16)
      concat    the direct sum of two N=32, chi=1024, d=2 chains (bond 2048)
      overlap   <X|Z> over the 64-site chi=256 benchmark chain and a second chain of its shape
      qr        Householder QR + thin Q of one 8192 x 4096 FP64 unfolding (the plain form's per-site step)
    Bytes are algorithmic (inputs read once, outputs written once); the
    ncu summaries under profiles/ give the DRAM counters of the same launches."""
    import numpy as np
    import torch

    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    rng = np.random.default_rng(SEED)

    def timed(fn):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    out = {"metric": "HBM-bound kernels: achieved GB/s of algorithmic bytes", "unit": "GB/s",
           "peak_hbm_gbs": hbm, "steps": args.steps, "warmup": max(args.warmup, 1), "kernels": {}}
    want = set(args.hbm_kernels.split(","))
    # contract
    if "contract" in want:
        X = L.as_device(rng.standard_normal((256, 2, 256)) / 16.0)
        W = L.as_device(rng.standard_normal((16, 2, 2, 16)) / 6.0)
        P = _ops.empty((256 * 16, 2, 256 * 16))
        ms = timed(lambda: L.call("sgt_site_contract_mpo_mps", L.ptr(X), 256, 2, 256, L.ptr(W), 16, 2, 16, L.ptr(P),
                                  L.stream_ptr()))
        by = 4096 * 2 * 4096 * 8 + X.numel() * 8 + W.numel() * 8
        out["kernels"]["contract_mpo_mps_kernel"] = {"ms": ms, "bytes": by, "gbs": by / ms / 1e6,
                                                     "frac": by / ms / 1e6 / hbm}
    # concat (config 4 shapes)
    if "concat" in want:
        A, B = config4_inputs()
        Ad = [L.as_device(c) for c in A]
        Bd = [L.as_device(c) for c in B]
        outs = _ops.concat(Ad, Bd)
        by = sum(o.numel() for o in outs) * 8 + sum(c.numel() for c in Ad + Bd) * 8
        # the kernel alone: outputs allocated once, one C-ABI call per step
        ap, _ap = L.ptr_array(Ad)
        bp, _bp = L.ptr_array(Bd)
        op, _op = L.ptr_array(outs)
        ash, _as = L.shape_array([_ops.shape3(c) for c in Ad])
        bsh, _bs = L.shape_array([_ops.shape3(c) for c in Bd])
        ms = timed(lambda: L.call("sgt_bond_concat_chain", len(Ad), ap, ash, bp, bsh, op, None, 0, L.stream_ptr()))
        del outs
        out["kernels"]["concat_kernel"] = {"ms": ms, "bytes": by, "gbs": by / ms / 1e6, "frac": by / ms / 1e6 / hbm,
                                           "note": "one launch for all 32 sites (zero blocks written too)"}
        del Ad, Bd
    # overlap over two 64-site chi=256 chains
    if "overlap" in want:
        Xh, _Wh = make_inputs()
        Yh = [rng.standard_normal(c.shape) / math.sqrt(CHI * D_PHYS) for c in Xh]
        Xd = [L.as_device(c) for c in Xh]
        Yd = [L.as_device(c) for c in Yh]
        ms = timed(lambda: _ops.overlap_device(Xd, Yd))
        by = sum(c.size for c in Xh + Yh) * 8
        fl = sum(2 * D_PHYS * (x.shape[0] * x.shape[2] * y.shape[2] + x.shape[0] * y.shape[0] * y.shape[2])
                 for x, y in zip(Xh, Yh))
        out["kernels"]["overlap_sweep"] = {"ms": ms, "bytes": by, "gbs": by / ms / 1e6, "frac": by / ms / 1e6 / hbm,
                                           "fp64_tflops": fl / ms / 1e9,
                                           "note": "a chain of FP64 GEMMs (2 per site, sequential): FP64-pipe and "
                                                   "latency bound, its bytes are small next to its flops"}
    # Householder QR of one 8192 x 4096 unfolding + thin Q (4096 columns)
    if "qr" in want:
        m, n = 8192, 4096
        A0 = torch.from_numpy(rng.standard_normal((m, n))).to("cuda")
        Aw = torch.empty_like(A0)
        Q = torch.empty((m, n), dtype=torch.float64, device="cuda")
        tau = torch.empty(n, dtype=torch.float64, device="cuda")
        ws = L.workspace(L.query("sgt_qr_workspace_size", m, n, n))

        def qr():
            Aw.copy_(A0)
            L.call("sgt_qr", L.ptr(Aw), m, n, n, L.ptr(tau), L.ptr(Q), n, L.ptr(ws), ws.numel(), L.stream_ptr())

        ms = timed(qr)
        fl = 2 * (2 * m * n * n - 2 * n ** 3 / 3)
        out["kernels"]["householder_qr_8192x4096"] = {
            "ms": ms, "fp64_tflops": fl / ms / 1e9,
            "note": "panel_kernel (cluster panel factorisation) + FP64 trailing updates; FP64-pipe bound"}
    out["value"] = next(iter(out["kernels"].values())).get("gbs") if out["kernels"] else None
    print(json.dumps(out))
    return 0


def run_serving(args):
    import numpy as np
    import torch

    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.serving import Job, RoundServer, latency_stats

    t_start = time.perf_counter()

    def log(msg):
        print("[serving %7.1f s] %s" % (time.perf_counter() - t_start, msg), file=sys.stderr, flush=True)

    rng = np.random.default_rng(11)
    srv = RoundServer(budget_bytes=120 << 30, slots=8)
    nsess = args.sessions
    for i in range(nsess):
        n = int(rng.integers(8, 129))
        d = int(rng.choice([2, 4]))
        chi = int(round(math.exp(rng.uniform(math.log(8), math.log(args.chi_max)))))
        D = int(rng.choice([4, 16]))
        dims = [1] + [chi] * (n - 1) + [1]
        X = [rng.standard_normal((dims[k], d, dims[k + 1])) / math.sqrt(chi * d) for k in range(n)]
        wd = [1] + [D] * (n - 1) + [1]
        W = [rng.standard_normal((wd[k], d, d, wd[k + 1])) / math.sqrt(D * d) for k in range(n)]
        srv.add_session("s%d" % i, mps=X, mpo=W)
        srv.sessions["s%d" % i]["chi"] = chi
    srv.start()
    log("%d sessions resident" % nsess)
    # seeded Poisson arrivals
    t = 0.0
    arrivals = []
    while t < args.duration:
        t += rng.exponential(1.0 / args.rate)
        arrivals.append(t)
    jobs = []
    t0 = time.perf_counter()
    for k, ta in enumerate(arrivals):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        sid = "s%d" % int(rng.integers(0, nsess))
        kind = ["round", "add_round", "overlap"][int(rng.integers(0, 3))]
        chi = srv.sessions[sid]["chi"]
        j = Job(kind=kind, session=sid, chi=chi, precision=PRECISIONS[args.precision], other=sid, job_id=k,
                arrival=t0 + ta)
        jobs.append(srv.submit(j))
    log("%d jobs submitted" % len(jobs))
    deadline = time.perf_counter() + args.drain
    for j in jobs:
        j.done.wait(max(0.0, deadline - time.perf_counter()))
    wall = time.perf_counter() - t0
    # the measurement: jobs finished by the drain deadline, over that wall time
    done = [j for j in jobs if j.done.is_set() and j.error is None]
    rejected = [j for j in jobs if j.done.is_set() and j.error is not None]
    log("drained: %d of %d done" % (len(done) + len(rejected), len(jobs)))
    stats = latency_stats(done)
    srv.stop(cancel_pending=True)
    out = {
        "metric": "serving jobs/s with p50/p99 latency", "value": len(done) / wall, "unit": "jobs/s",
        "n_gpus": 1, "higher_is_better": True,
        "dtype": "%s (round, add_round; no spectra), f64 (overlap)" % DTYPES[args.precision],
        "data": "synthetic seeded Poisson stream",
        "config": {"workload": "config5 stream: %.0f jobs/s for %.1f s, %d resident sessions, N~U[8,128], "
                               "d in {2,4}, chi log-uniform [8,%d], D in {4,16}, HBM budget 120 GB"
                               % (args.rate, args.duration, nsess, args.chi_max), "slots": 8},
        "submitted": len(jobs), "completed": len(done), "rejected_or_failed": len(rejected),
        "unfinished": len(jobs) - len(done) - len(rejected), "latency": stats, "wall_s": wall,
        "graph_replays": srv.replayed, "graphs": sum(1 for g in srv.graphs.values() if g is not None),
        "graph_bytes": srv.graph_bytes,
    }
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="syngular", choices=["syngular", "reference"])
    ap.add_argument("--precision", default="bf16x6", choices=sorted(PRECISIONS))
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed sweeps of the plain FP64 form (~62 s each)")
    ap.add_argument("--no-spectra-variant", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="config2", choices=["config2", "batched", "serving", "config4", "hbm"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--plain-sample", type=int, default=8)
    ap.add_argument("--rate", type=float, default=10.0)
    ap.add_argument("--duration", type=float, default=5.0)
    ap.add_argument("--sessions", type=int, default=16)
    ap.add_argument("--drain", type=float, default=120.0)
    ap.add_argument("--config4-spectra", action="store_true",
                    help="--workload config4: also run the rounding that returns every bond's spectrum")
    ap.add_argument("--split", default="",
                    help="CTAS,KTILES: the sliced GEMM's split-K shape (default: the library's 148,8)")
    ap.add_argument("--pchol", default="", choices=["", "cluster", "blocked"],
                    help="the BF16X6 form's pivoted Cholesky (default: the library's, cluster where it fits)")
    ap.add_argument("--purify-step", default="", choices=["", "warp", "block"],
                    help="the BF16X6 purification step: a warp per row or a block per row with 16-byte "
                         "accesses (default: the library's, block where the bond allows)")
    ap.add_argument("--graph-per-lane", type=int, default=4,
                    help="--workload batched: instances per lane in each captured graph (0 = one graph)")
    ap.add_argument("--hbm-kernels", default="contract,concat,overlap,qr",
                    help="--workload hbm: comma-separated subset of contract, concat, overlap, qr")
    ap.add_argument("--chi-max", type=int, default=512,
                    help="serving sessions: upper end of the log-uniform bond range")
    ap.add_argument("--sites", type=int, default=64, help="chain length (64 = the headline workload; shorter "
                    "chains only for profiling captures)")
    args = ap.parse_args()
    global N_SITES
    N_SITES = max(3, int(args.sites))
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "config4":
        return run_config4(args)
    if args.workload == "hbm":
        return run_hbm(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        return run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
