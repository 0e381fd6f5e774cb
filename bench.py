"""Lanczos throughput on one GB300 (or N independent replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload m573_n50k] [--precision mixed|fp64]

A bench step is one complete Lanczos run of the workload's length (300
bi-Lanczos steps for the default workload: 573 modes, 50 000 configurations,
no symmetry images, log-normal weights sigma 0.1), each Lanczos step two
operator applications (L and L^T) plus the float64 recurrence with full
re-biorthogonalisation, on a seeded synthetic ensemble with the workload's
shapes.  W runs are untimed, then K runs are timed with CUDA events on the
launching stream; `value` is Lanczos steps/s over them.  The ensemble
(2 x 50 000 x 573 float64 = 458 MB) is larger than L2, so no flush is needed
between steps; for workloads whose ensemble fits in L2 a 256 MB buffer is
written before each timed run.  One JSON line is printed by rank 0.

--impl reference times the reference's own CPU implementation of the same
step (its C kernels compiled from source when present, else the oracle's C
restatement) on the host cores, each step a bounded sample of the
configurations scaled to the full ensemble.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# hardware work queues for the batched leg's concurrent streams (read when the
# CUDA context is created; the default of 8 made streams share queues)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "Lanczos steps/s, M=576 N=50k: mixed vs FP64 GPU at ≤1e-4 rel spectral error"
UNIT = "steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5,
                    help="timed bench steps (one complete Lanczos run each)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="m573_n50k")
    ap.add_argument("--precision", default=None, choices=[None, "mixed", "fp64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--check-steps", type=int, default=None,
                    help="steps of the mixed-vs-float64 spectral check (default: the workload's)")
    ap.add_argument("--seeds", type=int, default=5,
                    help="ensembles / start vectors of the mixed-vs-float64 accuracy check")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the secondary measurements of the other operator paths")
    ap.add_argument("--qworkload", default="q444_nb12_n10k")
    ap.add_argument("--no-reorth", action="store_true",
                    help="plain recurrence (the reference default); without full "
                         "re-biorthogonalisation the spectral check is not reproducible "
                         "even between two float64 runs")
    return ap.parse_args()


def emit(line):
    """Print the JSON line last: C libraries loaded in this process (the
    reference's module prints its configuration split) buffer their stdout
    until exit, so flush the C stdio buffers first."""
    sys.stdout.flush()
    try:
        ctypes.CDLL(None).fflush(None)
    except (OSError, AttributeError):
        pass
    print(json.dumps(line), flush=True)


def job_throughput(ms_local, K, ws, device=None):
    """Whole-job steps/s of ws independent replicas that each ran K steps: the
    slowest rank's time (max over the process group) for ws x K steps.
    Returns (steps/s, that time in ms); ws = 1 needs no process group."""
    ms = float(ms_local)
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ws * K / (ms / 1e3), ms


def measured_peaks():
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(pk)) if os.path.exists(pk) else {}


def peaks_hbm():
    """Measured HBM copy bandwidth (GB/s), else the fallback 6800."""
    return measured_peaks().get("hbm_gbs", 6800.0)


L2_BYTES = 129e6


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms; the samples
    that arrive within the timed region (one interval either side) are kept."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def wait_first(self, n=3, timeout=3.0):
        """Block until n samples arrived: nvidia-smi's start-up (NVML
        initialisation, and whatever it still does right after its first
        sample) then lies before the timed region, not inside it."""
        t0 = time.time()
        while self.proc is not None and len(self.lines) < n and time.time() - t0 < timeout:
            time.sleep(0.01)

    def stop(self, t0=None, t1=None):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if t0 is not None and t1 is not None:
            inside = [x for x in lines if t0 - 0.02 <= x[0] <= t1 + 0.02]
            lines = inside if inside else lines
        for _, line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(name):
    from tdscha_gb300.synthetic import WORKLOADS, make_ensemble
    if name not in WORKLOADS:
        raise SystemExit("unknown workload %s (known: %s)" % (name, ", ".join(WORKLOADS)))
    spec = WORKLOADS[name]
    ens = make_ensemble(spec["M"], spec["N"], seed=2024, n_syms=spec["n_syms"],
                        rho_sigma=spec["rho_sigma"])
    return spec, ens


def identity_tables(M):
    return ([np.ones((1, 1, 1))] * M, [np.array([i], dtype=np.intc) for i in range(M)],
            np.arange(M, dtype=np.intc))


def sym_tables(ens):
    if ens.get("symmetries") is None:
        return identity_tables(ens["X"].shape[1])
    return ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]


# ----------------------------------------------------------------- CPU side
def cpu_sample_time(ens, n_cfg, n_threads, use_ref):
    """Seconds of one perturbation-average call over the first n_cfg configurations."""
    import oracle
    from tdscha_gb300.synthetic import random_R1, random_sym
    M = ens["X"].shape[1]
    syms, spaces, bid = sym_tables(ens)
    R1, Y1 = random_R1(M, 5), random_sym(M, 6, scale=1e-3)
    X, Y, rho = ens["X"][:n_cfg], ens["Y"][:n_cfg], ens["rho"][:n_cfg]
    t0 = time.perf_counter()
    if use_ref:
        import contextlib
        import io
        import sscha_HP_odd  # the reference's own C module, built from source
        f, d2v = np.zeros(M), np.zeros((M, M))
        with contextlib.redirect_stdout(io.StringIO()):
            sscha_HP_odd.GetPerturbAverageSym(X, Y, ens["w"], rho, R1, Y1, ens["T"], 1,
                                              syms[0].shape[0], syms,
                                              np.array([len(s) for s in spaces], np.intc),
                                              spaces, bid, f, d2v)
    else:
        oracle.perturb_averages(X, Y, ens["w"], rho, R1, Y1, ens["T"], 1, syms, spaces, bid,
                                n_threads=n_threads)
    return time.perf_counter() - t0


def cpu_impl():
    """('reference', 1 thread) when the reference's C module is importable here, else the port."""
    refdir = os.path.join(ROOT, "oracle", "_ref")
    if os.path.isdir(refdir):
        sys.path.insert(0, refdir)
        try:
            import sscha_HP_odd  # noqa: F401
            return "reference"
        except ImportError:
            pass
    return "port"


def cpu_baseline(ens, target_s, apps_per_step, force_port=False):
    import oracle
    oracle.build()
    N = ens["X"].shape[0]
    kind = "port" if force_port else cpu_impl()
    cores = 1 if kind == "reference" else (os.cpu_count() or 1)
    n0 = min(N, max(cores, 16))
    t0 = cpu_sample_time(ens, n0, cores, kind == "reference")
    n = int(min(N, max(n0, n0 * target_s / max(t0, 1e-6))))
    t = cpu_sample_time(ens, n, cores, kind == "reference") if n > n0 else t0
    per_app = t * N / n
    return {"value": 1.0 / (apps_per_step * per_app), "unit": UNIT, "cores": cores, "kind": kind,
            "sample": "perturbation averages over %d of %d configurations (%.1f s), scaled to "
                      "%d applications per step; recurrence not included" % (n, N, t, apps_per_step)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    spec, ens = workload(args.workload)
    import oracle
    oracle.build()
    kind = cpu_impl()
    cores = 1 if kind == "reference" else (os.cpu_count() or 1)
    N = ens["X"].shape[0]
    n0 = min(N, max(cores, 16))
    t0 = cpu_sample_time(ens, n0, cores, kind == "reference")
    # each step: a sample of about 2 s, scaled to the full step
    n = int(min(N, max(n0, n0 * 2.0 / max(t0, 1e-6))))
    for _ in range(args.warmup):
        cpu_sample_time(ens, n, cores, kind == "reference")
    tot = 0.0
    for _ in range(args.steps):
        tot += cpu_sample_time(ens, n, cores, kind == "reference")
    step_s = 2 * (tot / args.steps) * N / n
    value = 1.0 / step_s
    n_run = spec["steps"]
    sample = ("bi-Lanczos step = 2 perturbation-average calls; each timed sample runs one call "
              "over %d of %d configurations, scaled by N/%d and x2; a bench step (one %d-step "
              "run) is %d such Lanczos steps" % (n, N, n, n_run, n_run))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * step_s * n_run,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "M": spec["M"], "N": spec["N"],
                       "n_syms": spec["n_syms"],
                       "step": "one complete %d-step Lanczos run from the start vector; "
                               "value = Lanczos steps/s" % n_run,
                       "lanczos_steps_per_bench_step": n_run,
                       "lanczos": "bi-Lanczos (2 applications/step)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    emit(line)


# ------------------------------------------------------------------ GPU side
KERNEL_NAMES = {0: "stageA (V = D Y1 + quadratic forms)", 1: "row scalars", 2: "force average (+ W build, mixed)",
                3: "stageB (G = U^T W)", 4: "finalise", 5: "operand preparation"}


def run_ours(args):
    import torch
    import torch.distributed as dist
    from tdscha_gb300 import _native as nat
    from tdscha_gb300.synthetic import random_R1

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = nat.load()
    spec, ens = workload(args.workload)
    M, N, S = spec["M"], spec["N"], spec["n_syms"]
    n_run = spec["steps"]                  # Lanczos steps of one run (one bench step)
    prec_name = args.precision or "mixed"
    prec = nat.PREC_MIXED if prec_name == "mixed" else nat.PREC_FP64
    syms, spaces, bid = sym_tables(ens)
    # mixed: the ensemble held in 4-byte storage only (fp32 rows and fp16 limbs;
    # the float64 rows are released once the operands are built)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed="fp32" if prec_name == "mixed" else False)
    ctx.set_options(False, False, False, False, False, 0.0)     # bi-Lanczos (normal repr.)
    n_img, rows = ctx.layout()
    tuning = None
    if prec_name == "mixed":
        t_acc, t_split, t_ms = ctx.tuning()
        tuning = {"stage_a": "one accumulator, 128x192 tiles" if t_acc else
                  "two accumulators, 128x128 tiles", "stage_b_splits": t_split,
                  "application_ms_at_tuning": t_ms}
    P = ctx.P
    W, K = args.warmup, args.steps
    cap = n_run + 2
    dev = torch.device("cuda", local)
    ld = ctx.basis_ld()                  # rows padded to 256 bytes
    ctx.set_basis_ld(ld)
    Qd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    Pd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    psi = np.zeros(P)
    psi[:M] = random_R1(M, 11)
    first = torch.from_numpy(psi / np.sqrt(psi.dot(psi))).to(dev)
    Qd[0, :P].copy_(first)
    Pd[0, :P].copy_(first)
    hist = np.zeros(4 * cap)
    done = ctypes.c_int(0)
    conv = ctypes.c_int(0)
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    reorth = 0 if args.no_reorth else 1

    def one_run():
        """One complete n_run-step run from the start vector (the bench step)."""
        hist[:] = 0.0
        hist[3] = 1.0
        nat.check(lib.tdscha_lanczos_run(ctx.handle, Qd.data_ptr(), Pd.data_ptr(), cap, 0, n_run,
                                         0, prec, reorth, nat.dp(hist), ctypes.byref(done),
                                         ctypes.byref(conv), st))
        if conv.value or done.value != n_run:
            raise RuntimeError("Lanczos converged early (%d of %d steps)" % (done.value, n_run))

    # the clock sampler starts before the warm-up runs, so that its own
    # start-up cost is outside the timed region
    # an ensemble that fits in L2 stays resident across a run's steps (the
    # algorithm's reuse), but not across timed runs: a 256 MB buffer is
    # written before each run, inside the timed region.  The warm-up runs do
    # the same (the first fill in a process loads its kernel: ~250 ms)
    ens_bytes = 2 * rows * M * 8
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev) if ens_bytes < L2_BYTES else None
    clk = ClockSampler(local)
    clk.start()
    clk.wait_first()
    for _ in range(W):
        if flush is not None:
            flush.zero_()
        one_run()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_start = time.time()
    e0.record(stream)
    for _ in range(K):
        if flush is not None:
            flush.zero_()
        one_run()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop(t_start, time.time())
    ms = e0.elapsed_time(e1)
    value, ms = job_throughput(ms, K * n_run, ws, dev)
    if ws > 1:
        dist.barrier()

    # per-kernel device time: one more run with CUDA events around each kernel
    # of the perturbation averages (kept out of the timed runs)
    nat.check(lib.tdscha_ctx_profile(ctx.handle, 1))
    one_run()
    torch.cuda.synchronize()
    nat.check(lib.tdscha_ctx_profile(ctx.handle, 0))
    kern = {}
    for kid in range(8):
        tot, cnt = ctypes.c_double(0), ctypes.c_int(0)
        nat.check(lib.tdscha_ctx_profile_read(ctx.handle, kid, ctypes.byref(tot), ctypes.byref(cnt)))
        if cnt.value:
            kern[kid] = (tot.value, cnt.value)
    # the re-biorthogonalisation sweeps (ids 6: dots + coefficients, 7: update
    # + weight): each reads the stored pairs once, (k + 1) x 2 x P float64 at
    # step k, so a run's sweep reads sum_k (k + 1) 16 P bytes
    sweeps = None
    if 6 in kern and 7 in kern:
        sweep_bytes = sum((k + 1) * 16.0 * P for k in range(n_run))
        hbm = peaks_hbm()
        sweeps = {"basis_bytes_per_run_and_sweep": sweep_bytes}
        for kid, name in ((6, "dots"), (7, "update")):
            tot_ms = kern.pop(kid)[0]
            sweeps[name + "_ms_per_run"] = tot_ms
            sweeps[name + "_gbs"] = sweep_bytes / (tot_ms / 1e3) / 1e9
            sweeps[name + "_frac_of_measured_hbm"] = sweeps[name + "_gbs"] / hbm
    static = None
    if not args.no_rows and prec_name == "mixed":
        static = static_leg(lib, nat, ctx, M, S * N, dev,
                            lambda: nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"],
                                                ens["T"], syms, spaces, bid, with_mixed=False))
    ctx.close()
    R = N * S
    flops_app = 4.0 * R * M * M          # two GEMM stages of 2 R M^2 each
    # dominant kernel
    kid = max(kern, key=lambda k: kern[k][0]) if kern else None
    roof = None
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    # the mixed bi-Lanczos step runs L q and L^T p as one two-perturbation call
    # (one launch of each GEMM stage for both); the profiled run made
    # 2 n_run applications
    pair = prec_name == "mixed" and os.environ.get("TDSCHA_PAIR_APPLY", "1") != "0"
    ppl = 2 if pair else 1                  # perturbations per GEMM-stage launch
    if kid is not None:
        tot_ms, cnt = kern[kid]
        per_launch_s = tot_ms / cnt / 1e3
        if kid in (0, 3):
            work = 2.0 * R * M * M * ppl     # flops per launch of one GEMM stage
            achieved = work / per_launch_s / 1e12
            if prec_name == "fp64":
                peak, src = 1.25, "nominal GB300 FP64 1.25 TFLOP/s (not in MEASURED_PEAKS.json)"
            else:
                peak = peaks.get("bf16_tflops", 1900.0)
                src = "of measured bf16_tflops" if "bf16_tflops" in peaks else "of fallback"
            roof = {"bound": "tensor" if prec_name == "mixed" else "fp64", "kernel": KERNEL_NAMES[kid],
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": None, "peak_source": src,
                    "avg_launch_ms": tot_ms / cnt}
            if prec_name == "mixed":
                # three tensor products per K step (hi*hi, hi*lo, lo*hi) on the
                # padded mode count: the tensor-pipe work behind `achieved`
                Mp = ((M + 63) // 64) * 64
                roof["tensor_work_incl_split_tflops"] = 3 * 2.0 * R * Mp * Mp * ppl / per_launch_s / 1e12
                roof["frac_incl_split"] = roof["tensor_work_incl_split_tflops"] / peak
                # DRAM bytes per launch from the ncu captures of the same kernels
                # at N=20 000 (profiles/k_stageA_stageB_m573_n20k.md; one- and
                # two-perturbation launches), scaled by rows
                per_row = ({0: 147.2e6 / 20000, 3: 97.4e6 / 20000} if ppl == 1 else
                           {0: 252.26e6 / 20000, 3: 163.46e6 / 20000})[kid]
                if M == 573 and S == 1:
                    roof["traffic"] = per_row * R
                    roof["traffic_unit"] = "bytes per launch (ncu, scaled from N=20000)"
                    roof["hbm_frac"] = per_row * R / per_launch_s / 1e9 / peaks.get("hbm_gbs", 6800.0)
        else:
            nbytes = 2.0 * N * M * 8
            achieved = nbytes / per_launch_s / 1e9
            peak = peaks.get("hbm_gbs", 6800.0)
            roof = {"bound": "hbm", "kernel": KERNEL_NAMES[kid], "achieved": achieved, "peak": peak,
                    "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                    "avg_launch_ms": tot_ms / cnt}
    kernels = {KERNEL_NAMES[k]: {"ms_per_launch": v[0] / v[1], "launches": v[1],
                                 "perturbations_per_launch": ppl if (k != 4 or n_img == 1) else 1}
               for k, v in kern.items()}
    # kernels launched per Lanczos step.  One application: the averages and
    # the assemble (mixed: Y1 limbs read straight from psi, stage A, row
    # scalars, W build, stage B, finalisation; float64: psi unpack, stage A,
    # row scalars, force average, stage B, finalisation; with images on the
    # perturbation side the finalisation is three kernels and the float64 path
    # adds the image vectors and matrices).  One update pass per 1024 stored
    # pairs, here always one.
    per_app = 7 + ((3 if prec_name == "mixed" else 4) if n_img > 1 else 0)
    if pair:
        # one call for both: the Y1 preparation (with images: the Y1 unpack
        # and the image limbs), stage A, row scalars, W build, stage B, (no
        # images) the finalisation and the assemble once for both
        # perturbations; with images the three finalisation kernels per
        # perturbation
        per_step_ops = (2 + 4 + 6 + 1) if n_img > 1 else (1 + 4 + 1 + 1)
    else:
        per_step_ops = 2 * per_app
    # recurrence: dot + a, residuals + b/c, normalisation; re-biorthogonalisation:
    # dots, coefficients, update, weight
    per_step_rec = 3 + (4 if not args.no_reorth else 0)
    gpu_launches = K * n_run * (per_step_ops + per_step_rec)

    # float64 arm of the metric (same GPU, same runs) and the accuracy check
    fp64 = None
    check = None
    if prec_name == "mixed":
        fp64, check = fp64_arm_and_check(args, ens, spec, syms, spaces, bid, dev, local, rank)
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(ens, spec, prec_name, n_run, not args.no_reorth)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(ens, 15.0, 2)
    others = {}
    if static is not None:
        others["static"] = static
    if not args.no_rows:
        others["qspace"] = qspace_leg(args.qworkload, 20, 3, dev, peaks, with_cpu=not args.no_cpu)
        others["batched"] = batch_leg()
        others["learned_terminator"] = terminator_leg()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if prec_name == "fp64" else "fp16x3+f64",
                "data": "synthetic (seeded ensemble with the workload's shapes)",
                "precision": prec_name,
                "config": {"workload": args.workload, "M": M, "N": N, "n_syms": S,
                           "step": "one complete %d-step Lanczos run from the start vector; "
                                   "value = Lanczos steps/s over the K timed runs" % n_run,
                           "lanczos_steps_per_bench_step": n_run,
                           "lanczos": "bi-Lanczos (2 applications/step)",
                           "reorth": "none" if args.no_reorth else
                                     "full re-biorthogonalisation against the stored basis "
                                     "(float64 vectors, double-float sweeps)",
                           "symmetry_images": ("applied to the perturbation (%d), ensemble rows "
                                               "resident: %d" % (n_img, rows)) if S > 1 else "none",
                           "tuning": tuning,
                           "storage": ("ensemble resident in 4-byte storage only: fp32 rows "
                                       "and two-limb fp16 operands (float64 rows released "
                                       "after operand preparation)") if prec_name == "mixed"
                                      else "float64 rows",
                           "parallelism": "replicas" if ws > 1 else "single GPU",
                           "l2": ("inputs larger than L2 (ensemble %.0f MB)" % (ens_bytes / 1e6))
                                 if flush is None else
                                 ("ensemble %.0f MB fits in L2: a 256 MB buffer is written "
                                  "before each timed run, inside the timed region"
                                  % (ens_bytes / 1e6))},
                "roofline": roof, "kernels": kernels, "reorth_sweeps": sweeps,
                "cpu_baseline": cpu, "e2e": e2e,
                "fp64_gpu": fp64, "accuracy_vs_fp64": check,
                "clocks": clocks, "gpu_launches": gpu_launches, "other_paths": others,
                "flops_per_application": flops_app}
        emit(line)
    if ws > 1:
        dist.destroy_process_group()


def lanczos_coeffs(lib, nat, ctx, prec, n, dev, M, P, reorth=1, eps=0.0, r1_seed=11):
    """n bi-Lanczos steps from a seeded start vector; returns (a, b, c, seconds),
    the time by CUDA events on the launching stream around the whole run."""
    import torch
    from tdscha_gb300.synthetic import random_R1
    cap = n + 2
    ld = ctx.basis_ld()                  # rows padded to 256 bytes
    ctx.set_basis_ld(ld)
    Qd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    Pd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    psi = np.zeros(P)
    psi[:M] = random_R1(M, r1_seed)
    if eps:
        psi[:M] *= 1 + eps * np.random.default_rng(1).standard_normal(M)
    first = torch.from_numpy(psi / np.sqrt(psi.dot(psi))).to(dev)
    Qd[0, :P].copy_(first)
    Pd[0, :P].copy_(first)
    hist = np.zeros(4 * cap)
    hist[3] = 1.0
    done, conv = ctypes.c_int(0), ctypes.c_int(0)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    nat.check(lib.tdscha_lanczos_run(ctx.handle, Qd.data_ptr(), Pd.data_ptr(), cap, 0, n, 0, prec,
                                     reorth, nat.dp(hist), ctypes.byref(done), ctypes.byref(conv),
                                     stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    dt = e0.elapsed_time(e1) / 1e3
    k = done.value
    h = hist[: 4 * (k + 1)].reshape(-1, 4)
    nb = k - 1 if conv.value else k
    return h[:k, 0].copy(), h[:nb, 1].copy(), h[:nb, 2].copy(), dt


def spectral(a, b, c, wgrid, smear):
    """-Im G(w) of a bi-Lanczos run (continued fraction with terminator, in numpy)."""
    n = len(a)
    a_m, b_m, c_m = a[-1], b[-1], c[-1]
    dd = a_m - wgrid ** 2
    disc = dd ** 2 - 4 * b_m * c_m
    sq = np.sqrt(disc + 0j)
    gp, gm = (dd + sq) / (2 * b_m * c_m), (dd - sq) / (2 * b_m * c_m)
    g = np.where(np.abs(gp) < np.abs(gm), gp, gm)
    for i in range(n - 2, -1, -1):
        g = 1.0 / (a[i] - wgrid ** 2 + 2j * wgrid * smear - b[i] * c[i] * g)
    return -g.imag


def fp64_arm_and_check(args, ens, spec, syms, spaces, bid, dev, local, rank=0):
    """The float64 path on the same GPU and the mixed path's error against it.

    For seeds s = 0 .. n-1 (s = 0: the bench's ensemble and start vector;
    s > 0: ensemble seed 2024 + s, start-vector seed 11 + s) one float64 and
    one mixed run of the check length (the workload's full run, or for
    symmetric workloads the window in which two float64 runs reproduce each
    other) give the relative error of each coefficient a_n, b_n and of the
    spectral function on a 2000-point grid (0-700 cm^-1, 5 cm^-1 smearing).
    The float64 steps/s is the seed-0 run, timed by CUDA events like the
    mixed runs."""
    from tdscha_gb300 import _native as nat
    from tdscha_gb300.synthetic import make_ensemble
    lib = nat.load()
    M = spec["M"]
    n_check = args.check_steps if args.check_steps is not None else spec.get("check_steps",
                                                                             spec["steps"])
    reorth = 0 if args.no_reorth else 1
    w = np.linspace(0.0, 700.0, 2000) / 109691.40235
    sm = 5.0 / 109691.40235
    out, per_seed = {}, []
    for s in range(max(1, args.seeds)):
        e = ens if s == 0 else make_ensemble(M, spec["N"], seed=2024 + s, n_syms=spec["n_syms"],
                                             rho_sigma=spec["rho_sigma"])
        ctx64 = nat.Context(e["X"], e["Y"], e["w"], e["rho"], e["T"], syms, spaces, bid,
                            with_mixed=True)
        ctx64.set_options(False, False, False, False, False, 0.0)
        P = ctx64.P
        if s == 0:
            lanczos_coeffs(lib, nat, ctx64, nat.PREC_FP64, 1, dev, M, P, reorth)   # warm-up
        a64, b64, c64, t64 = lanczos_coeffs(lib, nat, ctx64, nat.PREC_FP64, n_check, dev, M, P,
                                            reorth, r1_seed=11 + s)
        amx, bmx, cmx, tmx = lanczos_coeffs(lib, nat, ctx64, nat.PREC_MIXED, n_check, dev, M, P,
                                            reorth, r1_seed=11 + s)
        ctx64.close()
        A64 = spectral(a64, b64, c64, w, sm)
        Amx = spectral(amx, bmx, cmx, w, sm)
        n = min(len(a64), len(amx))
        ra = np.abs(amx[:n] - a64[:n]) / np.abs(a64[:n])
        nb = min(len(b64), len(bmx))
        rb = np.abs(bmx[:nb] - b64[:nb]) / np.abs(b64[:nb])
        diff = np.abs(Amx - A64) / np.abs(A64).max()
        band = w >= sm          # frequencies the smearing resolves
        per_seed.append({"seed": s, "spectral_rel_err": float(diff[band].max()),
                         "at_cm": float(w[band][diff[band].argmax()] * 109691.40235),
                         "spectral_rel_err_full_grid": float(diff.max()),
                         "full_grid_at_cm": float(w[diff.argmax()] * 109691.40235),
                         "a_rel_err_max": float(ra.max()), "b_rel_err_max": float(rb.max()),
                         "fp64_run_s": t64, "mixed_run_s": tmx})
        if s == 0:
            out["fp64"] = {"value": n_check / t64, "unit": UNIT, "steps": n_check,
                           "timer": "CUDA events around a %d-step tdscha_lanczos_run" % n_check}
            out["full_run_steps_per_s"] = {"fp64": n_check / t64, "mixed": n_check / tmx}
    errs = [x["spectral_rel_err"] for x in per_seed]
    check = {"steps": n_check, "seeds": len(per_seed), "per_seed": per_seed,
             "spectral_rel_err": errs[0], "spectral_rel_err_max": float(max(errs)),
             "spectral_rel_err_median": float(np.median(errs)),
             "spectral_rel_err_full_grid_max": float(max(x["spectral_rel_err_full_grid"]
                                                         for x in per_seed)),
             "band": "spectral_rel_err: max |A_mixed - A_fp64| / max |A_fp64| over the grid "
                     "points w >= 5 cm^-1 (the smearing width; below it the reference's "
                     "smearing 2 i w eta vanishes and soft or unstable poles near w = 0, "
                     "small differences of large eigenvalues, are not broadened); "
                     "*_full_grid: all 2000 points",
             "a_rel_err_max": float(max(x["a_rel_err_max"] for x in per_seed)),
             "b_rel_err_max": float(max(x["b_rel_err_max"] for x in per_seed)),
             "all_within_1e-4": bool(max(errs) <= 1e-4),
             "grid": "2000 points 0-700 cm^-1, smearing 5 cm^-1, terminator on",
             "reorth": bool(reorth)}
    if spec["n_syms"] > 1:
        check["window"] = ("first %d steps: two float64 runs of this symmetric operator agree to "
                           "rounding there and part later (exactly degenerate eigenvalues)" % n_check)
    return out, check


def static_leg(lib, nat, ctx, M, R, dev, make_ctx64=None):
    """Static (Hessian) operator L1_static + anharmonic_static through
    tdscha_static_L: one StaticHessian / run_hessian_calculation matvec is M
    such applications.  Device time per application, mixed and float64 (on a
    float64 context from make_ctx64 when ctx holds 4-byte storage only)."""
    import torch
    Ps = M + M * (M + 1) // 2
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    g = torch.Generator(device=dev).manual_seed(5)
    out = {"what": "static operator (harmonic + anharmonic), batched rows of M + M(M+1)/2"}
    for name, prec, nvec in (("mixed", nat.PREC_MIXED, min(M, 96)), ("fp64", nat.PREC_FP64, 2)):
        own = prec == nat.PREC_FP64 and not ctx.fp64_storage
        if own:
            ctx = make_ctx64()
            ctx.set_options(False, False, False, False, False, 0.0)
        X = torch.randn((nvec, Ps), dtype=torch.float64, device=dev, generator=g)
        Y = torch.empty_like(X)
        nat.check(lib.tdscha_static_L(ctx.handle, 1, X.data_ptr(), Y.data_ptr(), 3, 1.0, prec, st))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nat.check(lib.tdscha_static_L(ctx.handle, nvec, X.data_ptr(), Y.data_ptr(), 3, 1.0, prec,
                                      st))
        e1.record(stream)
        nat.check(lib.tdscha_ctx_sync(ctx.handle, st))
        ms = e0.elapsed_time(e1) / nvec
        out[name] = {"ms_per_application": ms, "applications_per_s": 1e3 / ms,
                     "rows_timed": nvec, "matvec_s_at_M_rows": ms * M / 1e3,
                     "achieved_tflops": 4.0 * R * M * M / (ms / 1e3) / 1e12}
        if own:
            ctx.close()
    return out


def polarisation_starts(M, seed):
    """Nine synthetic R-sector start vectors standing for the 3 IR polarisations
    and the 6 independent Raman components of one structure: seeded random
    mode-space vectors (an effective-charge-like row per Cartesian direction,
    and products of two of them for the Raman components), unit norm."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((3, M))
    ir = [z[a] for a in range(3)]
    raman = [z[a] * z[b] for a in range(3) for b in range(a, 3)]
    return [v / np.linalg.norm(v) for v in ir + raman]


def batch_leg(n_steps=150, seed=31, n_real=36, n_q=28):
    """64 independent runs of uneven size advanced together
    (tdscha_lanczos_run_batch) against the same runs one after the other:
    n_real real-space runs, each on its own seeded ensemble (M log-uniform in
    [48, 384], N uniform in [2000, 40000]) from one of 3 IR / 6 Raman start
    vectors in turn, mixed precision with re-orthogonalisation; and n_q
    q-space runs at distinct q-points of a 4x4x4 grid (four 6-band ensembles
    of 5000 configurations, seven q-points each, Hermitian Lanczos with
    Gram-Schmidt, fp32 averages)."""
    import torch
    from tdscha_gb300.batch import run_batch
    from tdscha_gb300.DynamicalLanczos import Lanczos
    from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
    from tdscha_gb300.synthetic import make_ensemble, make_qspace_ensemble
    rng = np.random.default_rng(seed)
    specs = [(int(np.exp(rng.uniform(np.log(48), np.log(384)))), int(rng.uniform(2000, 40000)))
             for _ in range(n_real)]
    kinds = ["IR x", "IR y", "IR z", "Raman xx", "Raman xy", "Raman xz", "Raman yy", "Raman yz",
             "Raman zz"]
    ens = [make_ensemble(M, N, seed=seed + i, rho_sigma=0.1) for i, (M, N) in enumerate(specs)]
    starts = [polarisation_starts(M, seed + 100 + i)[i % 9] for i, (M, _) in enumerate(specs)]
    n_qens = 4
    qens = [make_qspace_ensemble((4, 4, 4), 6, 5000, seed=seed + 50 + i, dispersion=0.2)
            for i in range(n_qens)]
    qpts = [(i % n_qens, 1 + i) for i in range(n_q)]      # (ensemble, q-point index)

    def build():
        runs = []
        for i, e in enumerate(ens):
            lz = Lanczos.from_arrays(e["X"], e["Y"], e["w"], e["rho"], e["T"], use_wigner=False,
                                     precision="mixed")
            lz.init(use_symmetries=False)
            lz.full_reorth = True
            lz.prepare_perturbation(starts[i], masses_exp=0)
            runs.append(lz)
        for k, iq in qpts:
            e = qens[k]
            ql = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"],
                                           q_points=e["q"], precision="mixed")
            ql.init(use_symmetries=False)
            ql.prepare_mode_q(iq, 2)
            runs.append(ql)
        for r in runs:          # contexts, operands and first steps outside the timing
            r.run_FT(2, verbose=False)
        return runs

    seq = build()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in seq:
        r.run_FT(n_steps, verbose=False)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    for r in seq:
        r._invalidate()
    del seq
    bat = build()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_batch(bat, n_steps)
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    for r in bat:
        r._invalidate()
    total = n_steps * len(bat)
    return {"runs": len(bat), "real_space": [{"M": M, "N": N, "start": kinds[i % 9]}
                                             for i, (M, N) in enumerate(specs)],
            "qspace": "%d runs: q-points 1-%d of a 4x4x4 grid, 6 bands, N=5000" % (n_q, n_q),
            "steps_per_run": n_steps, "batched_steps_per_s": total / t_bat,
            "sequential_steps_per_s": total / t_seq, "speedup": t_seq / t_bat,
            "timer": "host wall clock, synchronised, contexts built beforehand"}


def terminator_leg():
    """The learned terminator (committed weights) on 20 fresh runs it was not
    trained on, at its training shapes (M log-uniform in [48, 160], N = 4000,
    320 Wigner steps with full re-orthogonalisation, mixed precision): 100
    measured steps extended to 320 against the 320-step run, and the operator
    applications the plain method needs to be as close (every step count from
    100 on)."""
    from tdscha_gb300.terminator import (DEFAULT_WEIGHTS, LearnedTerminator, evaluate,
                                         generate_runs)
    t0 = time.perf_counter()
    runs = generate_runs(20, 320, seed=7)
    t1 = time.perf_counter()
    term = LearnedTerminator()
    rep = evaluate(term, runs, 100, 320)
    rep["generate_s"] = t1 - t0
    rep["evaluate_s"] = time.perf_counter() - t1
    rep["runs_what"] = ("20 held-out seeded ensembles (M log-uniform in [48, 160], N = 4000, "
                        "anharmonic scale in [0.01, 0.1]), 320 Wigner steps with full "
                        "re-orthogonalisation, mixed precision")
    try:
        rep["training"] = json.loads(str(np.load(DEFAULT_WEIGHTS)["report"]))
    except (KeyError, ValueError):
        rep["training"] = None
    return rep


def qspace_leg(qname, K, W, dev, peaks, with_cpu=True):
    """q-space (Bloch basis) operator and Hermitian Lanczos, float64 complex:
    steps/s through QSpaceLanczos.run_FT, per-application device time of
    tdscha_qapply_full_L (CUDA events), FP64 roofline, CPU oracle sample."""
    import torch
    from tdscha_gb300 import _native as nat
    from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
    from tdscha_gb300.synthetic import QWORKLOADS, make_qspace_ensemble
    spec = QWORKLOADS[qname]
    e = make_qspace_ensemble(spec["dims"], spec["nb"], spec["N"], seed=7, rho_sigma=0.1,
                             dispersion=0.3)
    nb, n_q, N = spec["nb"], e["n_q"], spec["N"]
    lz = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"],
                                   q_points=e["q"])
    lz.init(use_symmetries=False)
    lz.prepare_mode_q(0, nb // 2)
    stream = torch.cuda.current_stream()
    lz.run_FT(W, verbose=False)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    lz.run_FT(K, verbose=False)
    e1.record(stream)
    torch.cuda.synchronize()
    steps_s = K / (e0.elapsed_time(e1) / 1e3)
    # one application at a time on device buffers
    ctx = lz._qcontext()
    P = ctx.P
    rng = np.random.default_rng(3)
    psi = torch.from_numpy(rng.standard_normal(2 * P)).to(dev)
    out = torch.empty_like(psi)
    lib = nat.load()
    st = stream.cuda_stream
    for _ in range(3):
        nat.check(lib.tdscha_qapply_full_L(ctx.handle, psi.data_ptr(), out.data_ptr(), st))
    torch.cuda.synchronize()
    reps = max(K, 10)
    e0.record(stream)
    for _ in range(reps):
        nat.check(lib.tdscha_qapply_full_L(ctx.handle, psi.data_ptr(), out.data_ptr(), st))
    e1.record(stream)
    torch.cuda.synchronize()
    app_s = e0.elapsed_time(e1) / 1e3 / reps
    n_pairs = ctx.n_pairs
    R = N
    L = n_q * nb
    # complex FMA = 8 flops: u = A x on every q (n_q nb^2), x^H u and u^H g (2 L),
    # d2v two FMAs per block element per row
    flops = R * (8.0 * n_q * nb * nb + 16.0 * L) + R * n_pairs * nb * nb * 16.0
    achieved = flops / app_s / 1e12
    out_d = {"workload": qname, "dims": list(spec["dims"]), "n_bands": nb, "N": N,
             "n_pairs": n_pairs, "psi_size": P,
             "lanczos_steps_per_s": steps_s,
             "lanczos": "Hermitian, Gram-Schmidt against all stored vectors (reference default)",
             "application_ms": app_s * 1e3,
             "roofline": {"bound": "fp64", "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
                          "frac": achieved / 1.25,
                          "peak_source": "nominal GB300 FP64 (not in MEASURED_PEAKS.json)",
                          "flops_per_application": flops},
             "ensemble_bytes": 2 * e["X_q"].nbytes}
    # the same operator with fp32 averages on the CUDA cores (precision mixed)
    lz.precision = "mixed"
    ctx = lz._qcontext()
    for _ in range(3):
        nat.check(lib.tdscha_qapply_full_L(ctx.handle, psi.data_ptr(), out.data_ptr(), st))
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        nat.check(lib.tdscha_qapply_full_L(ctx.handle, psi.data_ptr(), out.data_ptr(), st))
    e1.record(stream)
    torch.cuda.synchronize()
    app32 = e0.elapsed_time(e1) / 1e3 / reps
    lz.reset_q()
    lz.prepare_mode_q(0, nb // 2)
    lz.run_FT(W, verbose=False)
    torch.cuda.synchronize()
    e0.record(stream)
    lz.run_FT(K, verbose=False)
    e1.record(stream)
    torch.cuda.synchronize()
    out_d["mixed"] = {"application_ms": app32 * 1e3,
                      "lanczos_steps_per_s": K / (e0.elapsed_time(e1) / 1e3),
                      "achieved_tflops": flops / app32 / 1e12,
                      "what": "fp32 averages on the CUDA cores, float64 partial sums"}
    lz.precision = "fp64"
    # kernel polynomial method on the same operator: two moments per application
    from tdscha_gb300.QSpaceKPM import QSpaceKPM
    kpm = QSpaceKPM.from_qspace_lanczos(lz)
    kpm.prepare_mode_q(0, nb // 2)
    kpm.run_KPM(8, verbose=False)
    kpm.reset_q()
    kpm.prepare_mode_q(0, nb // 2)
    n_mom = 2 * K + 2
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kpm.run_KPM(n_mom, verbose=False)
    torch.cuda.synchronize()
    out_d["kpm"] = {"moments": n_mom, "moments_per_s": n_mom / (time.perf_counter() - t0),
                    "timer": "host wall clock around QSpaceKPM.run_KPM (one read-back)"}
    kpm._invalidate()
    if with_cpu:
        import oracle.qspace as oq
        ns = min(N, 400)
        R1 = np.zeros(nb, dtype=complex)
        R1[nb // 2] = 1
        blocks = [np.ones((nb, nb), dtype=complex)] * n_pairs
        pairs = [(q1, int(lz.q_pair_map[q1])) for q1 in range(n_q) if q1 <= lz.q_pair_map[q1]]
        t0 = time.perf_counter()
        oq.perturb_averages_qspace(e["X_q"][:, :ns], e["Y_q"][:, :ns], e["w_q"], e["rho"][:ns],
                                   R1, blocks, e["T"], True, 0, pairs)
        dt = (time.perf_counter() - t0) * N / ns
        out_d["cpu_baseline"] = {"value": 1.0 / dt, "unit": "applications/s", "cores": os.cpu_count(),
                                 "kind": "port",
                                 "sample": "oracle q-space averages (numpy) over %d of %d "
                                           "configurations, scaled" % (ns, N)}
    lz._invalidate()
    return out_d


def measure_e2e(ens, spec, prec_name, n_run, reorth):
    """Public API end to end, host buffers in and out: one bench step is
    Lanczos.from_arrays (ensemble upload) + init + prepare_perturbation +
    run_FT(n_run) + the continued fraction on 2000 frequencies (read back)."""
    import torch
    from tdscha_gb300.DynamicalLanczos import Lanczos
    from tdscha_gb300.synthetic import random_R1
    M = spec["M"]
    # the ensemble in pinned host memory (allocated and filled once, before
    # the timed runs): the upload inside each run is a DMA from pinned pages
    pinned = {}
    for k in ("X", "Y"):
        t = torch.empty(ens[k].shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = ens[k]
        pinned[k] = t

    def one(nsteps, phases=None):
        t0 = time.perf_counter()
        lanc = Lanczos.from_arrays(pinned["X"].numpy(), pinned["Y"].numpy(), ens["w"], ens["rho"],
                                   ens["T"], use_wigner=False, precision=prec_name)
        if ens.get("symmetries") is not None:
            lanc.init(use_symmetries=True,
                      symmetries=(ens["symmetries"], ens["degenerate_space"]))
        else:
            lanc.init(use_symmetries=False)
        lanc.full_reorth = reorth
        lanc.prepare_perturbation(random_R1(M, 11), masses_exp=0)
        lanc._context()          # the upload and operand preparation, timed apart
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        lanc.run_FT(nsteps, verbose=False)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        g = lanc.get_green_function_continued_fraction(np.linspace(0, 600, 2000) / 109691.40235,
                                                       smearing=5 / 109691.40235)
        t3 = time.perf_counter()
        lanc._invalidate()
        if phases is not None:
            phases.append((t1 - t0, t2 - t1, t3 - t2))
        return g

    one(min(n_run, 10))
    torch.cuda.synchronize()
    runs, phases = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        one(n_run, phases)
        torch.cuda.synchronize()
        runs.append(time.perf_counter() - t0)
    dt = float(np.median(runs))
    ph = np.median(np.array(phases), axis=0) * 1e3
    P = M + M * (M + 1)
    h2d = 2 * ens["X"].size * 8 + ens["w"].size * 8 + ens["rho"].size * 8 + P * 8
    d2h = 4 * n_run * 8 + 2 * 2000 * 8
    return {"value": n_run / dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "per": "bench step (one %d-step run)" % n_run,
            "runs_ms": [round(1e3 * r, 2) for r in runs], "stat": "median of 3 runs",
            "phases_ms": {"context (upload + operand preparation)": round(ph[0], 2),
                          "run_FT": round(ph[1], 2), "continued fraction": round(ph[2], 2)},
            "inputs": "ensemble X, Y in pinned host memory",
            "what": "Lanczos.from_arrays + init + prepare_perturbation + run_FT(%d) + "
                    "continued fraction on 2000 frequencies, ensemble upload included" % n_run}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
