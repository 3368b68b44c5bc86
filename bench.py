"""Benchmark of the HODLR hot path: factor + solve + logdet throughput at n = 2^16.

Workload (one step): n = 65536 points uniform on [0,1]^2 (seeded, k-d ordered), Matern nu=3/2
(variance 1, range 0.1) plus a 1e-3 nugget, Nystrom blocks of global rank 72, FixedLevel(8)
(256 leaves of 256 points): assemble, one matvec, symmetricfactorize!, a solve with 16 N(0,1)
right-hand sides and logdet.  The metric is steps per second.

Both arithmetic forms of the engine run on the same inputs: the mixed form (float-pair
factorisation on the FP32 pipe, FP64 assembly and matvec; `--precision mixed`, the default) and
the FP64 form.  The one selected is reported as `value`/`e2e`, the other beside it, with the
logdet and solve differences between them measured outside the timed regions.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision mixed|fp64]

--impl ours (default): the GB300 engine (libkmhodlr.so).  `value` is measured with inputs
resident in HBM through the device entry points; `e2e` through the host-pointer C ABI (pinned
host buffers, copies inside the timed region).  N > 1 runs N independent replicas (the path does
not shard; weak scaling).
--impl reference: the reference's CPU algorithm (the NumPy restatement in oracle/) on the host
cores, every timed step a full step of the same workload (n = 65536, FixedLevel(8)), with the
reference's own parallel structure (`plel = true`: its `mapf`/`foreachf` maps over leaves, blocks
and levels on a thread pool of all host threads, one BLAS thread per worker as the reference's
`BLAS.set_num_threads(1)`).  It re-executes itself with OPENBLAS_NUM_THREADS=1 when that is not
set, since the BLAS thread count is fixed when NumPy loads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "kernelmatrices.jl_gb300"))

N_POINTS = 65536
RANK = 72
LEVEL = 8            # FixedLevel(8)
NRHS = 16
PARAMS = (1.0, 0.1, 1e-3)
SEED = 20260101
WORKLOAD = "matern32_nystrom_n65536_r72_fixedlevel8_16rhs"


# ----------------------------------------------------------------------------------------------
# algorithmic work models
# ----------------------------------------------------------------------------------------------

def engine_flops(n: int, L: int, m0: int = 256, r: int = RANK) -> dict:
    """Algorithmic FP64 flops per launch class of the engine, for one step."""
    nleaf = 2 ** L
    nnode = nleaf - 1
    return {
        "leaf_chol": nleaf * m0 ** 3 / 3.0,
        "leaf_qr": nleaf * (2.0 * m0 * r * r - 2.0 * r ** 3 / 3.0),
        "node": (nnode - 1) * 7.0 * r ** 3 + 8.0 / 3.0 * r ** 3,
        # Phi panel solve (r columns) + forward and backward solve of NRHS columns
        "leaf_tri": nleaf * m0 * m0 * (r + 2 * NRHS),
    }


def leaf_tc_mma_flops(m: int, nleaf: int, r: int = RANK) -> dict:
    """bf16 tensor-core flops issued per step by the mixed form's tensor-core leaf stage (the
    launch grids of km_leaf_tc.cu for leaves of m points): every 128 x 64 tile of the block-column
    and update launches takes 28 slice products of K = 64, i.e. 28 x 2 x 128 x 64 x 64 flops; and
    the algorithmic float-pair flops those tiles stand for (2 flops per multiply-add of the
    block columns P = A X' and of the trailing updates C -= P P', lower triangles only)."""
    per_tile = 28 * 2 * 128 * 64 * 64
    tiles = 0
    alg = 0.0
    for c0 in range(0, m, 64):
        nb = min(64, m - c0)
        T = m - c0 - nb
        R = T + r
        RP = -(-R // 128) * 128
        tiles += RP // 128                       # block column
        alg += 2.0 * R * nb * nb
        for rt in range(-(-R // 128)):           # trailing update
            for ct in range(-(-T // 64)):
                rlast = min(128 * rt + 127, R - 1)
                if not (rlast < T and rlast < 64 * ct):
                    tiles += 1
        alg += 2.0 * nb * (T * (T + 1) / 2 + r * T)
    return {"mma_flops": nleaf * tiles * float(per_tile), "alg_flops": nleaf * alg}


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    return json.loads(f.read_text()) if f.exists() else {}


# ----------------------------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------------------------
# replicas (N > 1): the path does not shard, so every rank runs the whole workload on its own
# inputs; the timed region ends when the slowest rank ends
# ----------------------------------------------------------------------------------------------

def max_over_ranks(t_ms: float, dist=None, device: str = "cuda") -> float:
    """Duration of a timed region as the slowest rank saw it: an all-reduce MAX over the ranks
    of the process group (``dist`` = torch.distributed after init, None for one process).  The
    caller brackets the region with barriers on every rank."""
    if dist is None:
        return float(t_ms)
    import torch
    tt = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_value(world: int, steps: int, ms: float) -> float:
    """Whole-job steps per second: every one of ``world`` replicas ran ``steps`` steps within the
    slowest rank's ``ms`` milliseconds."""
    return world * steps / (ms / 1e3)


# ----------------------------------------------------------------------------------------------
# CPU legs (the oracle restatement of the reference)
# ----------------------------------------------------------------------------------------------

def line_config(world: int) -> dict:
    """The workload keys shared by the GPU line and the reference line."""
    return {"workload": WORKLOAD, "n": N_POINTS, "rank": RANK, "level": f"FixedLevel({LEVEL})", "nrhs": NRHS,
            "kernel": "matern32", "params": list(PARAMS),
            "l2": "inputs larger than L2 (leaf factors alone 268 MB)", "parallelism": f"replicas{world}",
            "calls": "km_assemble, km_matvec, km_factorize_solve (symmetricfactorize! + solve), km_logdet"}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_full_steps(steps: int, warmup: int, budget_s: float) -> dict:
    """Times full workload steps of the reference's CPU algorithm (oracle/): assemble, matvec,
    symmetricfactorize!, a 16-column solve and logdet at n = 65536, FixedLevel(8), with the
    reference's plel maps on a thread pool of all host threads.  Runs ``warmup`` untimed steps,
    then up to ``steps`` timed ones, fewer when the next one would end past ``budget_s`` seconds
    of timed work (at least one)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import hodlr_oracle as O
    from kmhodlr.data import uniform_points
    nt = host_threads()
    pool = ThreadPoolExecutor(nt) if nt > 1 else None
    pts = uniform_points(N_POINTS, SEED)
    rng = np.random.default_rng(SEED + 100)
    rhs = rng.standard_normal((N_POINTS, NRHS))
    xv = rng.standard_normal((N_POINTS, 1))

    def step():
        K = O.KernelMatrix(pts, pts, np.array(PARAMS), O.KERNEL_MATERN32)
        HK = O.build_hodlr(K, 0.0, RANK, O.FixedLevel(LEVEL), nystrom=True, pool=pool)
        O.hodlr_mul(HK, xv)
        O.symmetricfactorize(HK, pool=pool)
        O.hodlr_ldiv(HK, rhs)
        return O.hodlr_logdet(HK)

    for _ in range(warmup):
        step()
    times = []
    ld = None
    while len(times) < steps:
        if times and sum(times) + statistics.mean(times) > budget_s:
            break
        t0 = time.perf_counter()
        ld = step()
        times.append(time.perf_counter() - t0)
    if pool is not None:
        pool.shutdown()
    return {"times": times, "threads": nt, "logdet": ld, "blas": os.environ.get("OPENBLAS_NUM_THREADS")}


def _single_blas_env() -> dict:
    env = dict(os.environ)
    for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        env[k] = "1"
    return env


REF_SAMPLE = ("every timed step is a full workload step (n=65536 FixedLevel(8), Nystrom rank 72, 16 RHS: "
              "assemble, matvec, symmetricfactorize!, solve, logdet) of the reference algorithm restated in "
              "oracle/, with the reference's plel=true maps on a thread pool of all host threads and one BLAS "
              "thread per worker")


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    if os.environ.get("OPENBLAS_NUM_THREADS") != "1":
        # the BLAS thread count is read when NumPy loads: start over with one BLAS thread
        os.execve(sys.executable, [sys.executable, str(Path(__file__).resolve()), *sys.argv[1:]],
                  _single_blas_env())
    # warm-up: the algorithm has no caches to warm; two steps page the code and data in
    warm = min(args.warmup, 2)
    res = cpu_full_steps(args.steps, warm, budget_s=args.ref_budget)
    per_step = statistics.mean(res["times"])
    value = 1.0 / per_step
    steps = len(res["times"])
    sample = REF_SAMPLE
    if steps < args.steps:
        sample += f"; {steps} of the {args.steps} requested steps timed (time budget {args.ref_budget:.0f} s)"
    out = {"metric": "HODLR factor+solve+logdet/s", "value": value, "unit": "steps/s", "n_gpus": world,
           "steps": steps, "warmup": warm, "ms_per_step": per_step * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": line_config(world), "precision": "fp64",
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "steps/s", "cores": res["threads"], "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "step_s": res["times"], "logdet": res["logdet"]}
    print(json.dumps(out), flush=True)


def cpu_baseline_line(steps: int = 2, warmup: int = 1) -> dict:
    """The cpu_baseline object of the GPU line: a bounded sample of the reference arm (two full
    workload steps after one untimed step), run in a child process with one BLAS thread."""
    cmd = [sys.executable, str(Path(__file__).resolve()), "--impl", "reference", "--steps", str(steps),
           "--warmup", str(warmup), "--ref-budget", "60"]
    env = _single_blas_env()
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run(cmd, env=env, capture_output=True, text=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not line:
        return {"value": None, "unit": "steps/s", "cores": host_threads(), "kind": "port",
                "sample": f"reference leg failed: {r.stderr.strip()[-200:]}"}
    ref = json.loads(line[-1])
    cb = dict(ref["cpu_baseline"])
    cb["sample"] = f"{ref['steps']} timed full steps after {ref['warmup']} untimed; " + cb["sample"]
    return cb


# ----------------------------------------------------------------------------------------------
# GPU leg
# ----------------------------------------------------------------------------------------------

def run_ours(args, rank: int, world: int, local_rank: int):
    import torch
    import kmhodlr
    from kmhodlr import _lib as L
    from kmhodlr.data import uniform_points

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (no CPU fallback)")
    dev = local_rank
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    lib = L.load()
    n = N_POINTS
    pts = uniform_points(n, SEED + rank)
    rng = np.random.default_rng(SEED + 100 + rank)
    rhs = rng.standard_normal((n, NRHS))
    xv = rng.standard_normal((n, 1))

    # pinned host buffers (column-major = contiguous columns)
    h_pts = torch.from_numpy(pts.reshape(-1)).pin_memory()
    h_rhs = torch.from_numpy(np.ascontiguousarray(rhs.T).reshape(-1)).pin_memory()
    h_x = torch.from_numpy(xv.reshape(-1).copy()).pin_memory()
    h_sol = torch.empty(n * NRHS, dtype=torch.float64).pin_memory()
    h_y = torch.empty(n, dtype=torch.float64).pin_memory()
    d_pts = h_pts.cuda()
    d_rhs = h_rhs.cuda()
    d_x = h_x.cuda()
    d_sol = torch.empty(n * NRHS, dtype=torch.float64, device="cuda")
    d_y = torch.empty(n, dtype=torch.float64, device="cuda")
    params = np.array(PARAMS, dtype=np.float64)
    pp = params.ctypes.data_as(C.POINTER(C.c_double))

    def check(h, rc):
        if rc != 0:
            raise RuntimeError(lib.km_last_error(h).decode())

    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def run_form(prec: int, sample_clocks: bool) -> dict:
        cfg = L.KmConfig(device=dev, precision=prec, hbm_budget_fraction=0.8, refine_max_iter=0, refine_tol=0.0)
        h = C.c_void_p()
        rc = lib.km_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise SystemExit(f"km_create failed ({rc})")
        lib.km_set_stream(h, C.c_void_p(stream.cuda_stream))
        logdet = C.c_double()

        def step_dev():
            check(h, lib.km_assemble_dev(h, C.c_void_p(d_pts.data_ptr()), n, L.KM_KERNEL_MATERN32, pp, 3,
                                         L.KM_METHOD_NYSTROM, 0.0, RANK, L.KM_LEVEL_FIXED, LEVEL))
            check(h, lib.km_matvec_dev(h, C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()), 1))
            # symmetricfactorize! then K \ b as one call (the forward half of the solve overlaps the
            # factorisation; the same bits as km_factorize + km_solve_dev)
            check(h, lib.km_factorize_solve_dev(h, C.c_void_p(d_rhs.data_ptr()), C.c_void_p(d_sol.data_ptr()),
                                                NRHS))
            check(h, lib.km_logdet(h, C.byref(logdet)))

        def step_e2e():
            check(h, lib.km_assemble(h, dp(h_pts), n, L.KM_KERNEL_MATERN32, pp, 3, L.KM_METHOD_NYSTROM, 0.0, RANK,
                                     L.KM_LEVEL_FIXED, LEVEL))
            check(h, lib.km_matvec(h, dp(h_x), dp(h_y), 1))
            check(h, lib.km_factorize_solve(h, dp(h_rhs), dp(h_sol), NRHS))
            check(h, lib.km_logdet(h, C.byref(logdet)))

        def timed(fn, steps):
            barrier()
            st0 = L.KmStats()
            lib.km_get_stats(h, C.byref(st0))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
            st1 = L.KmStats()
            lib.km_get_stats(h, C.byref(st1))
            t = max_over_ranks(e0.elapsed_time(e1), dist)
            return t, st1.kernel_launches - st0.kernel_launches

        # clocks are sampled from the start of the warm-up through the end of the timed region
        # (a 10-step timed region is shorter than two sampling periods)
        clocks = ClockSampler(dev) if sample_clocks else None
        if clocks:
            clocks.start()
        for _ in range(args.warmup):
            step_dev()
        ms, launches = timed(step_dev, args.steps)
        clk = clocks.stop() if clocks else None
        sol = d_sol.cpu().numpy().copy()
        ld = logdet.value
        ms_e2e, _ = timed(step_e2e, args.steps)
        lib.km_profile_enable(h, 1)
        timed(step_dev, args.steps)
        prof = {}
        for ci, name in enumerate(L.PROF_CLASSES):
            tot, cnt = C.c_double(), C.c_int64()
            lib.km_profile_get(h, ci, C.byref(tot), C.byref(cnt))
            if cnt.value:
                prof[name] = {"ms": tot.value / args.steps, "launches": cnt.value // args.steps}
        lib.km_profile_enable(h, 0)
        lib.km_destroy(h)
        return {"ms": ms, "launches": launches, "clk": clk, "ms_e2e": ms_e2e, "prof": prof, "sol": sol, "logdet": ld}

    head_prec = L.KM_PREC_MIXED if args.precision == "mixed" else L.KM_PREC_FP64
    other_prec = L.KM_PREC_FP64 if head_prec == L.KM_PREC_MIXED else L.KM_PREC_MIXED
    head = run_form(head_prec, True)
    other = run_form(other_prec, False)
    f64 = other if head_prec == L.KM_PREC_MIXED else head
    mix = head if head_prec == L.KM_PREC_MIXED else other
    fp64_peak = kmhodlr.probe_fp64_tflops(dev)
    fp32_peak = kmhodlr.probe_fp32_tflops(dev)

    def form_summary(fm):
        return {"value": replica_value(world, args.steps, fm["ms"]), "ms_per_step": fm["ms"] / args.steps,
                "e2e_value": replica_value(world, args.steps, fm["ms_e2e"]), "kernel_ms_per_step": fm["prof"]}

    step_ms = head["ms"] / args.steps
    value = replica_value(world, args.steps, head["ms"])
    e2e_value = replica_value(world, args.steps, head["ms_e2e"])
    flops = engine_flops(n, LEVEL)
    prof = head["prof"]
    dom = max((k for k in prof if k in flops), key=lambda k: prof[k]["ms"], default=None)
    roof = None
    if dom:
        achieved = flops[dom] / (prof[dom]["ms"] * 1e-3) / 1e12
        traffic = None
        tf = ROOT / "profiles" / "ncu_traffic.json"
        if tf.exists():
            traffic = json.loads(tf.read_text()).get(f"{args.precision}:{dom}")
        if head_prec == L.KM_PREC_MIXED:
            # one float-pair multiply-add (2 algorithmic flops) costs 18 FP32 instructions, i.e. 9 FP32
            # FMA slots (18 FP32 flops) per algorithmic flop pair: peak = FP32 flop rate / 18
            peak = fp32_peak / 18.0
            src = ("FP32 FMA rate measured live by km_probe_fp32_tflops / 18 (a float-pair multiply-add is 18 "
                   "FP32 instructions for 2 algorithmic flops)")
            bound = "fp32"
        else:
            peak = fp64_peak
            src = "FP64 FMA rate measured live by km_probe_fp64_tflops"
            bound = "fp64"
        roof = {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic,
                "per_launch_ms": prof[dom]["ms"] / max(prof[dom]["launches"], 1), "peak_source": src,
                "fp64_peak_tflops": fp64_peak, "fp32_peak_tflops": fp32_peak}
    # the tensor-core leaf kernels (mixed form): issued bf16 work against the measured bf16 peak
    roof_tc = None
    if head_prec == L.KM_PREC_MIXED and "leaf_tc" in prof:
        tcw = leaf_tc_mma_flops(n // 2 ** LEVEL, 2 ** LEVEL)
        sec = prof["leaf_tc"]["ms"] * 1e-3
        pk = measured_peaks()
        peak_tc = pk.get("bf16_tflops")
        ach = tcw["mma_flops"] / sec / 1e12
        roof_tc = {"kernel": "leaf_tc (k_lc_trsm, k_lc_update)", "bound": "tensor", "achieved": ach,
                   "peak": peak_tc, "unit": "TFLOP/s", "frac": (ach / peak_tc) if peak_tc else None,
                   "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peak_tc else "absent",
                   "issued_bf16_tflop_per_step": tcw["mma_flops"] / 1e12,
                   "algorithmic_float_pair_tflops": tcw["alg_flops"] / sec / 1e12,
                   "ms_per_step": prof["leaf_tc"]["ms"], "launches": prof["leaf_tc"]["launches"]}
    accuracy = {"logdet_abs_err_mixed_vs_fp64": abs(mix["logdet"] - f64["logdet"]),
                "solve_rel_err_mixed_vs_fp64": float(np.linalg.norm(mix["sol"] - f64["sol"]) /
                                                     np.linalg.norm(f64["sol"])),
                "targets": {"logdet_abs": 1e-6, "solve_rel": 1e-8}}
    out = {"metric": "HODLR factor+solve+logdet/s", "value": value, "unit": "steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if head_prec == L.KM_PREC_FP64 else "f32x2+f64",
           "data": "synthetic",
           "config": line_config(world), "precision": args.precision,
           "e2e": {"value": e2e_value, "unit": "steps/s",
                   "h2d_bytes_per_step": int((2 * n + n + NRHS * n) * 8),
                   "d2h_bytes_per_step": int((n + NRHS * n + 1) * 8)},
           "gpu_launches": int(head["launches"]),
           "clocks": head["clk"],
           "roofline": roof,
           "roofline_tensor": roof_tc,
           "fp64_form": form_summary(f64),
           "mixed_form": form_summary(mix),
           "mixed_speedup_vs_fp64": f64["ms"] / mix["ms"],
           "accuracy": accuracy,
           "logdet": head["logdet"]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_line()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ----------------------------------------------------------------------------------------------
# further workloads (not the headline line): batched likelihoods, serving, ACA at 2^18
# ----------------------------------------------------------------------------------------------

def _loguniform(rng, lo, hi, size):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=size))


def batch_problems(count: int, lo: int, hi: int, seed: int):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    rng = np.random.default_rng(seed)
    ns = np.round(_loguniform(rng, lo, hi, count)).astype(np.int64)
    rhos = _loguniform(rng, 0.02, 0.3, count)
    return [K.Problem(uniform_points(int(n), seed + 1 + b), rng.standard_normal(int(n)), (1.0, float(rho), 1e-3))
            for b, (n, rho) in enumerate(zip(ns, rhos))]


def run_batch(args):
    """256 independent Nystrom likelihood problems (n log-uniform in [2^10, 2^15], range
    log-uniform in [0.02, 0.3], nugget 1e-3, rank 72, LogLevel(8), 72 Rademacher probes): NLL and
    the 3-parameter stochastic gradient of every problem per step."""
    import torch
    import kmhodlr as K
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (no CPU fallback)")
    probs = batch_problems(256, 2 ** 10, 2 ** 15, SEED)
    prec = L_prec(args.precision)
    out_forms = {}
    for label, nw in (("pool", args.workers), ("one_stream", 1)):
        eng = K.BatchEngine(nworkers=nw, precision=prec)
        for _ in range(args.warmup if label == "pool" else 1):
            eng.nll_grad(probs, K.Matern32(), RANK, K.LogLevel(8), nprobe=72, seed=SEED)
        steps = args.steps if label == "pool" else 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            nll, grad, status = eng.nll_grad(probs, K.Matern32(), RANK, K.LogLevel(8), nprobe=72, seed=SEED)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        out_forms[label] = {"workers": nw, "s_per_batch": dt, "problems_per_s": len(probs) / dt}
        eng.close()
    v = out_forms["pool"]["problems_per_s"]
    ns = [len(p.y) for p in probs]
    out = {"metric": "batched NLL+gradient problems/s", "value": v, "unit": "problems/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * out_forms["pool"]["s_per_batch"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if prec == 0 else "f32x2+f64", "data": "synthetic",
           "config": {"workload": "batch256_matern32_nystrom_r72_loglevel8_72probes", "problems": len(probs),
                      "n_min": int(min(ns)), "n_max": int(max(ns)), "n_total": int(sum(ns)),
                      "precision": args.precision},
           "e2e": {"value": v, "unit": "problems/s", "h2d_bytes_per_step": int(sum(24 * n for n in ns)),
                   "d2h_bytes_per_step": int(len(probs) * 32),
                   "note": "the batch call takes host inputs; value and e2e are the same host-to-host timing"},
           "forms": out_forms, "speedup_pool_vs_one_stream": v / out_forms["one_stream"]["problems_per_s"]}
    print(json.dumps(out), flush=True)


def run_grad(args):
    """One likelihood request of the serving mix at its largest size: assemble (Nystrom rank 72,
    LogLevel(8)), factorise and evaluate NLL + stochastic gradient with 72 seeded probes for one
    dataset of n points (Matern nu = 3/2, range 0.1, nugget 1e-3); both precision forms, phase
    times from host timers around the calls (each call ends with a device synchronisation)."""
    import torch
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (no CPU fallback)")
    n = args.grad_n
    pts = uniform_points(n, SEED + 21)
    y = np.random.default_rng(SEED + 22).standard_normal(n)
    km = K.KernelMatrix(pts, pts, PARAMS, K.Matern32())
    forms = {}
    head = L_prec(args.precision)
    for prec in (head, 1 - head):
        times = []
        for it in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hk = K.KernelHODLR(km, 0.0, RANK, K.LogLevel(8), nystrom=True, precision=prec)
            K.symmetricfactorize(hk)
            t1 = time.perf_counter()
            nll, g = hk.nll_grad_seeded(y, 72, SEED + it)
            t2 = time.perf_counter()
            if it >= args.warmup:
                times.append((t1 - t0, t2 - t1))
            del hk
        a = float(np.mean([t[0] for t in times]))
        b = float(np.mean([t[1] for t in times]))
        forms["mixed" if prec == 1 else "fp64"] = {"requests_per_s": 1.0 / (a + b), "ms_per_request": 1e3 * (a + b),
                                                  "assemble_factor_ms": 1e3 * a, "nll_grad_ms": 1e3 * b,
                                                  "nll": nll, "grad": [float(v) for v in g]}
    h = forms[args.precision]
    out = {"metric": "NLL+gradient requests/s", "value": h["requests_per_s"], "unit": "requests/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": h["ms_per_request"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if head == 0 else "f32x2+f64", "data": "synthetic",
           "config": {"workload": f"nllgrad_matern32_nystrom_n{n}_r72_loglevel8_72probes", "n": n,
                      "params": list(PARAMS)},
           "precision": args.precision, "forms": forms}
    print(json.dumps(out), flush=True)


def L_prec(name: str) -> int:
    return 1 if name == "mixed" else 0


def serve_once(args, precision: int) -> dict:
    """One Poisson request stream against a fresh server of the given precision form."""
    import kmhodlr as K
    rng = np.random.default_rng(SEED + 7)
    nreq = args.requests
    srv = K.Server(K.Matern32(), RANK, K.LogLevel(8), nworkers=args.workers, precision=precision,
                   hbm_budget_fraction=0.8)
    facs = batch_problems(8, 2 ** 12, 2 ** 18, SEED + 11)
    fids = []
    for p in facs:
        r = srv.wait(srv.submit_factor(p))
        if r.status != 0:
            raise SystemExit(f"factor build failed: {r.status}")
        fids.append((r.factor_id, len(p.y)))
    pool = batch_problems(64, 2 ** 12, 2 ** 18, SEED + 13)   # datasets of the likelihood requests
    kinds = rng.uniform(size=nreq) < 0.2
    gaps = rng.exponential(1.0 / args.rate, size=nreq)
    rhs_cache = {}
    tickets = []
    t_start = time.perf_counter()
    next_t = t_start
    for q in range(nreq):
        next_t += gaps[q]
        d = next_t - time.perf_counter()
        if d > 0:
            time.sleep(d)
        if kinds[q]:
            tickets.append(srv.submit_nll_grad(pool[q % len(pool)], nprobe=72, seed=q))
        else:
            fid, n = fids[int(rng.integers(len(fids)))]
            k = int(rng.integers(1, 33))
            key = (n, k)
            if key not in rhs_cache:
                rhs_cache[key] = np.asfortranarray(np.random.default_rng(k).standard_normal((n, k)))
            tickets.append(srv.submit_solve(fid, rhs_cache[key]))
    t_offered = time.perf_counter() - t_start
    statuses = [srv.wait(t).status for t in tickets]
    t_end = time.perf_counter()
    st = srv.stats()
    srv.close()
    ok = sum(1 for x in statuses if x == 0)
    return {"served_per_s": ok / (t_end - t_start), "offered_per_s": nreq / t_offered, "wall_s": t_end - t_start,
            "requests": nreq, "ok": ok, "latency_ms": {"p50": st.p50_ms, "p99": st.p99_ms, "mean": st.mean_ms},
            "completed": int(st.completed), "failed": int(st.failed), "rejected": int(st.rejected),
            "peak_bytes": int(st.peak_bytes), "budget_bytes": int(st.budget_bytes)}


def run_serve(args):
    """Serving: Poisson arrivals at 200 requests/s, 10^4 requests; a request is an NLL + gradient
    of a new dataset (n log-uniform in [2^12, 2^18], 72 probes) with probability 0.2, else 1-32
    solves on one of 8 resident factors (built before the timed region).  80 % HBM budget.  The
    same stream runs against the mixed form and the FP64 form; `value` is the selected form."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (no CPU fallback)")
    head = L_prec(args.precision)
    forms = {}
    for prec in (head, 1 - head):
        forms["mixed" if prec == 1 else "fp64"] = serve_once(args, prec)
    h = forms[args.precision]
    out = {"metric": "served requests/s", "value": h["served_per_s"], "unit": "requests/s", "n_gpus": 1,
           "steps": args.requests, "warmup": 0, "ms_per_step": 1e3 * h["wall_s"] / args.requests,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if head == 0 else "f32x2+f64", "data": "synthetic",
           "config": {"workload": "serve_poisson_matern32_nystrom_r72_loglevel8", "rate_per_s": args.rate,
                      "requests": args.requests, "nll_fraction": 0.2, "resident_factors": 8, "workers": args.workers,
                      "hbm_budget_fraction": 0.8},
           "precision": args.precision,
           "latency_ms": h["latency_ms"], "offered_rate_per_s": h["offered_per_s"],
           "forms": forms}
    print(json.dumps(out), flush=True)


def aca_dense_subsample(nugget: float) -> dict:
    """The ACA pipeline at n = 2^14 (the configuration's kernel, tol and LogLevel) against the
    dense FP64 Cholesky factorisation of the exact kernel matrix (torch on the GPU, the checker):
    the compression error of the matvec, logdet and 8-column solve, and the solve's residual
    against the compressed and the exact matrix."""
    import torch
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n = 2 ** 14
    params = (1.0, 0.05, nugget)
    pts = uniform_points(n, SEED + 5)
    rhs = np.asfortranarray(np.random.default_rng(SEED + 6).standard_normal((n, 8)))
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, params, K.Matern32()), 1e-8, 0, K.LogLevel(8), nystrom=False)
    y_h = hk @ rhs
    K.symmetricfactorize(hk)
    x_h = hk.ldiv(rhs)
    ld_h = hk.logdet()
    res_h = float(np.linalg.norm(hk @ x_h - rhs) / np.linalg.norm(rhs))
    x = torch.as_tensor(pts, dtype=torch.float64, device="cuda")
    z = (3.0 ** 0.5) * torch.cdist(x, x) / params[1]
    kd = params[0] * (1.0 + z) * torch.exp(-z)
    kd.diagonal().add_(params[2])
    b = torch.as_tensor(rhs, device="cuda")
    L = torch.linalg.cholesky(kd)
    ld_d = float(2.0 * torch.log(torch.diagonal(L)).sum())
    x_d = torch.cholesky_solve(b, L).cpu().numpy()
    y_d = (kd @ b).cpu().numpy()
    res_d = float(torch.linalg.norm(kd @ torch.as_tensor(x_h, device="cuda") - b) / torch.linalg.norm(b))
    out = {"n": n, "params": list(params), "matvec_relerr": float(np.linalg.norm(y_h - y_d) / np.linalg.norm(y_d)),
           "logdet": ld_h, "logdet_dense": ld_d, "logdet_abserr": abs(ld_h - ld_d),
           "solve_relerr": float(np.linalg.norm(x_h - x_d) / np.linalg.norm(x_d)),
           "residual_compressed": res_h, "residual_exact": res_d}
    del kd, L, z, x
    torch.cuda.empty_cache()
    return out


def run_aca(args):
    """ACA assembly and general factorisation at n = 2^18 (range 0.05, nugget 1e-4, tol 1e-8,
    LogLevel(8) => 10 levels), 8 right-hand sides, logdet.  ``--aca-nugget`` changes the nugget:
    at n = 2^18 the ACA error of the widest blocks is of the order of 1e-4, so the compressed
    matrix with the config's nugget is not positive definite (the factorisation raises
    PosDefException, as the reference's would)."""
    import torch
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (no CPU fallback)")
    n = args.aca_n
    pts = uniform_points(n, SEED + 3)
    rhs = np.asfortranarray(np.random.default_rng(SEED + 4).standard_normal((n, 8)))
    km = K.KernelMatrix(pts, pts, (1.0, 0.05, args.aca_nugget), K.Matern32())
    times = []
    for it in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hk = K.KernelHODLR(km, 1e-8, 0, K.LogLevel(8), nystrom=False)
        t1 = time.perf_counter()
        K.symmetricfactorize(hk)
        t2 = time.perf_counter()
        x = hk.ldiv(rhs)
        ld = hk.logdet()
        t3 = time.perf_counter()
        if it >= args.warmup:
            times.append((t1 - t0, t2 - t1, t3 - t2))
        ranks = hk.block_ranks()
        del hk
    a, f, s = (float(np.mean([t[i] for t in times])) for i in range(3))
    tot = a + f + s
    out = {"metric": "ACA HODLR assemble+factor+solve/s", "value": 1.0 / tot, "unit": "steps/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"aca_matern32_n{n}_tol1e-8_loglevel8_8rhs", "n": n, "levels": int(np.log2(n)) - 8,
                      "params": [1.0, 0.05, args.aca_nugget]},
           "phase_s": {"assemble": a, "factorize": f, "solve_logdet": s},
           "ranks": {"max": int(ranks.max()), "mean": float(ranks.mean()), "blocks": int(ranks.size)},
           "logdet": ld, "dense_subsample": aca_dense_subsample(args.aca_nugget)}
    print(json.dumps(out), flush=True)


def main():
    global N_POINTS, LEVEL, WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=900.0,
                    help="reference arm: seconds of timed CPU work after which no further step starts")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed",
                    help="form reported as `value` (the other form is reported beside it)")
    ap.add_argument("--workload", choices=["c2", "batch", "serve", "aca", "grad"], default="c2",
                    help="c2: the headline factor+solve+logdet step; batch / serve / aca / grad: the other forms")
    ap.add_argument("--workers", type=int, default=8, help="batch / serve: concurrent handles")
    ap.add_argument("--requests", type=int, default=10000, help="serve: number of requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: Poisson arrival rate (1/s)")
    ap.add_argument("--aca-n", type=int, default=2 ** 18, help="aca: number of points")
    ap.add_argument("--aca-nugget", type=float, default=1e-4, help="aca: nugget of the Matern kernel")
    ap.add_argument("--grad-n", type=int, default=2 ** 18, help="grad: number of points")
    ap.add_argument("--n", type=int, default=N_POINTS,
                    help="c2: number of points (a smaller case of the same leaf size for profiling)")
    ap.add_argument("--level", type=int, default=LEVEL, help="c2: FixedLevel of the smaller case")
    args = ap.parse_args()
    if (args.n, args.level) != (N_POINTS, LEVEL):
        N_POINTS, LEVEL = args.n, args.level
        WORKLOAD = f"matern32_nystrom_n{N_POINTS}_r{RANK}_fixedlevel{LEVEL}_{NRHS}rhs"
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "aca":
        run_aca(args)
    elif args.workload == "grad":
        run_grad(args)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
