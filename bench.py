"""Benchmark: factor + PCG to a 1e-8 relative residual on one GB300.

A step is one numeric factorisation of the workload's matrix (same pattern,
values resident on the device) followed by one PCG solve to ||r||/||b|| <=
1e-8.  `value` is solves per second over the K timed steps (whole job: N
independent replicas under torchrun, max time over ranks).  `e2e` is the same
step through the C ABI with host buffers (values and right-hand side copied
in, solution copied out inside the timed region).  The default precision is
mixed (FP32 factor and apply, FP64 PCG); the plain FP64 GPU path is timed on
the same workload in the same run (`plain_fp64`).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c2]
                    [--precision fp64|mixed] [--impl ours|reference]

The CPU baseline (and the reference arm) is the CPU oracle -- the FP64
restatement of the reference's factor + PCG path (the reference itself
cannot be built: CHOLMOD, CSparse, Boost and LAPACKE are absent) -- timed on
the host cores with threaded BLAS.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (description, generator spec, nrhs, factor parameters beyond the reference driver's defaults)
    "c1": ("2D 5-point Poisson 128x128, Dirichlet, seed 0; ND leaves <= 64, separators above 16 columns compressed "
           "(HODLR leaves <= 32), ranks <= 32 with oversampling 10",
           ("diffusion", 2, 128, 0.0, 0), 1,
           dict(nd_leaf=64, max_dense_block=16, max_diag_block=32, rank_cap=32, oversampling=10)),
    "c2": ("3D 7-point variable-coefficient diffusion 64^3, log-normal sigma=1 seed 1, harmonic faces",
           ("diffusion", 3, 64, 1.0, 1), 1, dict()),
    "c3": ("3D Q1 hex linear elasticity 48^3 elements, E=1 nu=0.3, x=0 face clamped, seed 2; ranks <= 64",
           ("elasticity", 48, 0, 0, 2), 1, dict(rank_cap=64)),
    "c4": ("2D 5-point variable-coefficient 1024^2, log-normal sigma=2 seed 3, 64 RHS",
           ("diffusion", 2, 1024, 2.0, 3), 64, dict()),
    # serving stream (run_serving): a pool of matrices, Poisson arrivals
    "c5": ("serving stream: 2000 requests, Poisson arrivals at 200/s, pool of 2D grids (side 64-1024) and 3D "
           "grids (side 16-96), log-normal sigma=1 seed per matrix id, 1-16 RHS per request, to 1e-8",
           None, 0, dict()),
    # a smaller case of c2 for multi-pass ncu captures (a few hundred MB on the device)
    "c2s": ("3D 7-point variable-coefficient diffusion 40^3, log-normal sigma=1 seed 1, harmonic faces",
            ("diffusion", 3, 40, 1.0, 1), 1, dict()),
}


def config_params(cfg):
    return dict(CONFIGS[cfg][3])


def make_problem(cfg, cpu_only=False):
    """The workload's system.  cpu_only builds it with the CPU oracle's copy
    of the generators (the same arrays), so that the CPU arm never loads the
    GPU library."""
    _, spec, nrhs, _ = CONFIGS[cfg]
    if cpu_only:
        from oracle import pyoracle as gen
    else:
        import rank_structured_cholesky_gb300 as gen
    if spec[0] == "diffusion":
        _, dim, nx, sigma, seed = spec
        return gen.diffusion(dim, nx, sigma=sigma, seed=seed, nrhs=nrhs)
    _, ne, _, _, seed = spec
    return gen.elasticity(ne, seed=seed, nrhs=nrhs)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup(gpus):
    if gpus <= 1 and "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", gpus))
    backend = "nccl" if os.environ.get("RSCHOL_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
    dist.init_process_group(backend=backend)
    return rank, world, dist


def reduce_max(dist, value, device):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_oracle_solve(prob, params):
    from oracle import pyoracle as po
    t0 = time.perf_counter()
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, params)
    t1 = time.perf_counter()
    assert F.factor() == 0
    t2 = time.perf_counter()
    x, it, rec, true = F.pcg(prob.rhs[0], 1e-8, 10000)
    t3 = time.perf_counter()
    return dict(symbolic_s=t1 - t0, factor_s=t2 - t1, pcg_s=t3 - t2, iterations=it, true_residual=true)


def run_reference(args):
    rank, world, dist = dist_setup(args.gpus)
    if rank != 0:
        return 0
    if args.config == "c5":
        stream = serving_stream(args.requests, 200.0, seed=5)
        probs, rhs = serving_pool([m for m in range(len(SERVING_POOL)) if SERVING_POOL[m][1] <= 32], cpu_only=True)
        small = tuple(np.array(v)[[i for i in range(len(stream[0])) if int(stream[1][i]) in probs]] for v in stream)
        vals = [serving_cpu_sample(small, probs, rhs, 20.0) for _ in range(max(1, args.steps // 5))]
        cpu = vals[-1]
        print(json.dumps({"impl": "reference", "metric": "serving: solve requests/s to 1e-8 relative residual",
                          "value": cpu["value"], "unit": "requests/s", "n_gpus": args.gpus, "steps": len(vals),
                          "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64", "data": "synthetic", "config": {"workload": "c5"}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "requests/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return 0
    prob = make_problem(args.config, cpu_only=True)
    params = config_params(args.config)
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_oracle_solve(prob, params)
    times = []
    last = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        last = cpu_oracle_solve(prob, params)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": "factor+PCG solves/s to 1e-8 relative residual", "value": value,
        "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.config, "description": CONFIGS[args.config][0], "n": prob.n,
                   "params": params, "parallelism": "single process, threaded BLAS"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "full %s solve per step (symbolic + factor + PCG to 1e-8)" % args.config},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "iterations": last["iterations"], "true_residual": last["true_residual"],
        "factor_s": last["factor_s"], "pcg_s": last["pcg_s"], "symbolic_s": last["symbolic_s"],
        "p50_ms": 1e3 * statistics.median(times),
        "p99_ms": 1e3 * float(np.percentile(times, 99)),
    }
    print(json.dumps(line), flush=True)
    return 0


def traffic_from_profiles(kernel, workload="c2"):
    """(dram bytes per launch, algorithmic bytes per launch) of `kernel` from
    the committed ncu summary, either None when absent."""
    path = os.path.join(ROOT, "profiles", "%s_%s.md" % (kernel, workload))
    got = {}
    try:
        for line in open(path):
            for key in ("traffic_bytes_per_launch", "algorithmic_bytes_per_launch"):
                if line.startswith(key + ":"):
                    got[key] = float(line.split(":", 1)[1])
    except OSError:
        pass
    return got.get("traffic_bytes_per_launch"), got.get("algorithmic_bytes_per_launch")


def timed_solves(lib, rs, torch, prob, params, precision, device, local, steps, warmup, dist, step_timing):
    """K timed factor + PCG steps (device-resident inputs) for one precision."""
    ctx = rs.Context(**params, precision=precision, device=local)
    t0 = time.perf_counter()
    F = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(lib.rschol_stream(ctx.h), device=device)
    nrhs = prob.nrhs
    d_vals = torch.from_numpy(prob.vals).to(device)
    d_b = torch.from_numpy(np.ascontiguousarray(prob.rhs[:nrhs])).to(device)
    d_x = torch.zeros_like(d_b)
    infos = (rs.PcgInfo * nrhs)()
    schedule = F.tune_schedule(2)   # the factor's schedule, timed once before any timed work
    if nrhs > 1:   # tile shapes of the batched apply, likewise
        F.autotune(nrhs)
    torch.cuda.synchronize()

    def refactor():
        st = lib.rschol_refactor_device(F.h, d_vals.data_ptr())
        if st != 0:
            raise rs.RscholError(st, ctx.last_error())

    def pcg():
        st = lib.rschol_pcg_device(F.h, d_b.data_ptr(), d_x.data_ptr(), nrhs, 1e-8, 10000, infos)
        if st not in (0, 5):
            raise rs.RscholError(st, ctx.last_error())

    for _ in range(warmup):
        refactor()
        pcg()
    torch.cuda.synchronize()
    barrier(dist)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * steps + 1)]
    counters = np.zeros(24)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        ev[0].record(stream)
        for k in range(steps):
            refactor()
            ev[2 * k + 1].record(stream)
            pcg()
            ev[2 * k + 2].record(stream)
        torch.cuda.synchronize()
    if step_timing:
        # the same K steps again with a CUDA event around every factor step
        # (per-kind device time, GEMM flops): the roofline and the breakdown
        # come from this pass, the reported time from the plain one above
        lib.rschol_step_timing(F.h, 1, None)
        for k in range(steps):
            refactor()
            pcg()
        torch.cuda.synchronize()
        lib.rschol_step_timing(F.h, 0, counters.ctypes.data)
    barrier(dist)
    step_ms = [ev[2 * k].elapsed_time(ev[2 * k + 2]) for k in range(steps)]
    factor_ms = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(steps)]
    pcg_ms = [ev[2 * k + 1].elapsed_time(ev[2 * k + 2]) for k in range(steps)]
    total_s = reduce_max(dist, ev[0].elapsed_time(ev[2 * steps]) / 1e3, device)
    return dict(ctx=ctx, F=F, stream=stream, d_b=d_b, infos=infos, setup_s=setup_s, schedule=schedule, step_ms=step_ms,
                factor_ms=factor_ms, pcg_ms=pcg_ms, total_s=total_s, clocks=clocks.summary(), counters=counters,
                iterations=[infos[k].iterations for k in range(nrhs)],
                true_residual=max(infos[k].true_residual for k in range(nrhs)))


def run_ours(args):
    import torch
    import rank_structured_cholesky_gb300 as rs

    rank, world, dist = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    lib = rs.load_library()
    prob = make_problem(args.config)
    n, nrhs = prob.n, prob.nrhs

    if args.profile:
        # ncu --profile-from-start off: capture exactly the K steps
        ctx = rs.Context(**config_params(args.config), precision=args.precision, device=local)
        F = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz)
        d_vals = torch.from_numpy(prob.vals).to(device)
        d_b = torch.from_numpy(np.ascontiguousarray(prob.rhs[:nrhs])).to(device)
        d_x = torch.zeros_like(d_b)
        infos = (rs.PcgInfo * nrhs)()

        def step_device():
            lib.rschol_refactor_device(F.h, d_vals.data_ptr())
            lib.rschol_pcg_device(F.h, d_b.data_ptr(), d_x.data_ptr(), nrhs, 1e-8, 10000, infos)

        for _ in range(args.warmup):
            step_device()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for _ in range(args.steps):
            step_device()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        if rank == 0:
            print(json.dumps({"profiled_steps": args.steps, "config": args.config, "precision": args.precision,
                              "iterations": [infos[k].iterations for k in range(nrhs)],
                              "fused_cholesky": F.describe().get("fused_cholesky")}), flush=True)
        return 0

    params = config_params(args.config)
    main = timed_solves(lib, rs, torch, prob, params, args.precision, device, local, args.steps, args.warmup, dist,
                        True)
    F, ctx, stream = main["F"], main["ctx"], main["stream"]
    stats = F.stats()
    desc = F.describe()

    # end to end through the C ABI with host buffers (copies inside the timed
    # region, from and to pinned host memory)
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64).pin_memory()
        arr = t.numpy()
        arr[...] = a
        return t, arr
    _pv, h_vals = pinned(prob.vals)
    _pb, h_b = pinned(np.ascontiguousarray(prob.rhs[:nrhs]))
    _px, h_x = pinned(np.zeros((nrhs, n)))
    infos = (rs.PcgInfo * nrhs)()

    def step_e2e():
        st = lib.rschol_refactor(F.h, rs._dp(h_vals))
        if st != 0:
            raise rs.RscholError(st, ctx.last_error())
        st = lib.rschol_pcg(F.h, rs._dp(h_b), rs._dp(h_x), nrhs, 1e-8, 10000, infos)
        if st not in (0, 5):
            raise rs.RscholError(st, ctx.last_error())

    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    torch.cuda.synchronize()
    barrier(dist)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_e2e()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_s = reduce_max(dist, e0.elapsed_time(e1) / 1e3, device)

    # phase breakdown (apply, SpMV) and launch counts
    phase = profile_phases(lib, F, ctx, stream, main["d_b"], nrhs, torch)

    # the plain FP64 path on the same workload, for the mixed-precision speed-up
    plain = None
    if args.precision == "mixed" and not args.no_fp64_plain:
        pf = timed_solves(lib, rs, torch, prob, params, "fp64", device, local, args.steps, args.warmup, dist, False)
        plain = {"value": world * args.steps / pf["total_s"], "unit": "solves/s",
                 "ms_per_step": 1e3 * pf["total_s"] / args.steps,
                 "factor_ms": statistics.median(pf["factor_ms"]), "pcg_ms": statistics.median(pf["pcg_ms"]),
                 "p50_ms": statistics.median(pf["step_ms"]), "p99_ms": float(np.percentile(pf["step_ms"], 99)),
                 "iterations": pf["iterations"] if nrhs > 1 else pf["iterations"][0],
                 "true_residual": pf["true_residual"], "clocks": pf["clocks"]}
        # the mixed results against the FP64 path (which matches the FP64 oracle to 1e-7 per apply):
        # one preconditioner application and the PCG solution, same right-hand side
        b0 = np.ascontiguousarray(prob.rhs[0])
        z_mixed, z_fp64 = F.apply(b0), pf["F"].apply(b0)
        x_mixed, _ = F.pcg(b0, eps=1e-8)
        x_fp64, _ = pf["F"].pcg(b0, eps=1e-8)
        plain["mixed_vs_fp64"] = {
            "apply_rel_error": float(np.linalg.norm(z_mixed - z_fp64) / np.linalg.norm(z_fp64)),
            "solution_rel_error": float(np.linalg.norm(x_mixed - x_fp64) / np.linalg.norm(x_fp64)),
            "note": "relative 2-norm differences on rhs[0]; both solves stop at ||r||/||b|| <= 1e-8"}
        # mixed precision with the root separator's dense Cholesky in FP64: its cost and its error
        rf = timed_solves(lib, rs, torch, prob, dict(params, root_fp64=1), "mixed", device, local, args.steps,
                          args.warmup, dist, False)
        z_root = rf["F"].apply(b0)
        x_root, _ = rf["F"].pcg(b0, eps=1e-8)
        plain["mixed_root_fp64"] = {
            "value": world * args.steps / rf["total_s"], "unit": "solves/s",
            "factor_ms": statistics.median(rf["factor_ms"]), "pcg_ms": statistics.median(rf["pcg_ms"]),
            "iterations": rf["iterations"] if nrhs > 1 else rf["iterations"][0],
            "true_residual": rf["true_residual"],
            "apply_rel_error_vs_fp64": float(np.linalg.norm(z_root - z_fp64) / np.linalg.norm(z_fp64)),
            "solution_rel_error_vs_fp64": float(np.linalg.norm(x_root - x_fp64) / np.linalg.norm(x_fp64))}
        # mixed precision with the split products as BF16 hi/lo pairs: its cost and its error
        bf = timed_solves(lib, rs, torch, prob, dict(params, schur_bf16=1), "mixed", device, local, args.steps,
                          args.warmup, dist, False)
        z_bf = bf["F"].apply(b0)
        x_bf, _ = bf["F"].pcg(b0, eps=1e-8)
        plain["mixed_schur_bf16"] = {
            "value": world * args.steps / bf["total_s"], "unit": "solves/s",
            "factor_ms": statistics.median(bf["factor_ms"]), "pcg_ms": statistics.median(bf["pcg_ms"]),
            "iterations": bf["iterations"] if nrhs > 1 else bf["iterations"][0],
            "true_residual": bf["true_residual"],
            "apply_rel_error_vs_fp64": float(np.linalg.norm(z_bf - z_fp64) / np.linalg.norm(z_fp64)),
            "solution_rel_error_vs_fp64": float(np.linalg.norm(x_bf - x_fp64) / np.linalg.norm(x_fp64))}
        del pf, rf, bf

    hbm, bf16, src = peaks()
    if rank == 0:
        total_s = main["total_s"]
        value = world * args.steps / total_s
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            cores = os.cpu_count()
            res = cpu_oracle_solve(prob, params)
            t = res["symbolic_s"] + res["factor_s"] + res["pcg_s"]
            cpu = {"value": 1.0 / t, "unit": "solves/s", "cores": cores, "kind": "port",
                   "sample": "one full %s solve (symbolic + FP64 factor + PCG to 1e-8, %d iterations) with the "
                             "CPU oracle, threaded BLAS" % (args.config, res["iterations"]),
                   "factor_s": res["factor_s"], "pcg_s": res["pcg_s"], "iterations": res["iterations"]}
        # rooflines of the dominant kernel (the fused blocked Cholesky / TRSM
        # launches, chol_fused_kernel, 22.5% of the c2 launch list) and of the
        # remaining GEMM launches, timed with CUDA events around every factor
        # step of the instrumented pass of the K timed steps
        c = main["counters"]
        step_total_ms = sum(main["step_ms"])

        # context for FP32 SIMT work: 152 SMs x 128 FP32 lanes x 2 flops x the SM clock sampled in the run
        sm_mhz = (main["clocks"] or {}).get("sm_mhz") or 2070.0
        fp32_nominal = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12

        def roofline(kernel, ms, launches, flops, traffic, traffic_source):
            achieved = flops / (ms * 1e-3) / 1e12 if ms > 0 else 0.0
            return {"bound": "tensor", "kernel": kernel, "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                    "frac": achieved / bf16, "fp32_simt_nominal": fp32_nominal,
                    "frac_of_fp32_simt_nominal": achieved / fp32_nominal,
                    "traffic": traffic, "traffic_source": traffic_source,
                    "peak_source": src, "flops_per_launch": flops / max(launches, 1),
                    "launch_ms": ms / max(launches, 1), "launches_per_step": launches / args.steps,
                    "share_of_step_time": ms / step_total_ms if step_total_ms else None}

        # the fused Cholesky's algorithmic bytes: every job's lower front region
        # (rows x first nUpd columns) read once and written once per launch
        fc = desc.get("fused_cholesky", {})
        chol_bytes = fc.get("algorithmic_bytes", 0.0) / max(fc.get("launches", 1), 1)
        t_small, a_small = traffic_from_profiles("chol_fused_kernel", "c2s")
        # the c2s capture's dram bytes per algorithmic byte, applied to this
        # workload's algorithmic bytes per launch (traffic grows with the fronts)
        chol_traffic = t_small / a_small * chol_bytes if (t_small and a_small) else None
        roof = roofline("chol_fused_kernel (blocked Cholesky and TRSM chains of a level, FP32 SIMT, ticketed tiles)",
                        c[21], c[22], c[23], chol_traffic,
                        "profiles/chol_fused_kernel_c2s.md: dram bytes per algorithmic byte of the c2s launches, "
                        "times this workload's algorithmic bytes per launch")
        chol_launch_ms = roof["launch_ms"]
        roof["algorithmic_bytes_per_launch"] = chol_bytes
        roof["hbm_achieved_gbs"] = chol_bytes / (chol_launch_ms * 1e-3) / 1e9 if chol_launch_ms else None
        roof["hbm_frac"] = roof["hbm_achieved_gbs"] / hbm if roof["hbm_achieved_gbs"] else None
        roof["traffic_over_algorithmic"] = t_small / a_small if (t_small and a_small) else None
        t_gemm, _ = traffic_from_profiles("gemm_tc_kernel", "c2s")
        roof_gemm = roofline("factor GEMMs (gemm_kernel SIMT and gemm_tc_kernel tcgen05)", c[0], c[1], c[2],
                             t_gemm, "profiles/gemm_tc_kernel_c2s.md: average DRAM bytes of the c2s GEMM launches, "
                             "not scaled")
        apply_bytes = phase["apply_bytes"]
        its = main["iterations"][0]
        pcg_bytes = its * (apply_bytes + phase["spmv_bytes"] + 8.0 * 10 * n)
        pcg_med = statistics.median(main["pcg_ms"])
        roof_pcg = {"bound": "hbm", "kernel": "PCG iteration (SpMV + preconditioner apply + vector updates)",
                    "achieved": pcg_bytes / (pcg_med * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                    "frac": pcg_bytes / (pcg_med * 1e-3) / 1e9 / hbm, "peak_source": src,
                    "bytes_per_iteration": pcg_bytes / its, "apply_bytes": apply_bytes,
                    "apply_ms": phase["apply_ms"], "spmv_ms": phase["spmv_ms"]}
        line = {
            "metric": "factor+PCG solves/s to 1e-8 relative residual", "value": value, "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32 factor / f64 pcg",
            "data": "synthetic",
            "config": {"workload": args.config, "description": CONFIGS[args.config][0], "n": n, "nrhs": nrhs,
                       "params": params, "precision": args.precision, "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (factor arena %.0f MB)" % (stats["device_bytes"] / 1e6)},
            "e2e": {"value": world * args.steps / e2e_s, "unit": "solves/s",
                    "h2d_bytes_per_step": int(prob.vals.nbytes + h_b.nbytes),
                    "d2h_bytes_per_step": int(h_x.nbytes)},
            "gpu_launches": int(args.steps * (phase["factor_launches"] + phase["pcg_launches"])),
            # the dominant kernel's roofline: the fused Cholesky unless the tuned schedule
            # runs none of it (per-panel launches), then the factor's GEMM launches
            "roofline": roof if c[22] > 0 else dict(roof_gemm, note="no fused Cholesky launches in the tuned "
                                                        "schedule: the GEMM launches are the dominant kernel"),
            "roofline_fused_cholesky": roof, "roofline_gemm": roof_gemm,
            "roofline_pcg": roof_pcg,
            "cpu_baseline": cpu,
            "clocks": main["clocks"],
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "iterations": main["iterations"] if nrhs > 1 else main["iterations"][0],
            "true_residual": main["true_residual"],
            "factor_ms": statistics.median(main["factor_ms"]), "pcg_ms": statistics.median(main["pcg_ms"]),
            "apply_ms": phase["apply_ms"], "spmv_ms": phase["spmv_ms"], "setup_s": main["setup_s"],
            "symbolic_s": stats["symbolic_s"],
            "p50_ms": statistics.median(main["step_ms"]), "p99_ms": float(np.percentile(main["step_ms"], 99)),
            "factor_gflop": stats["factor_flops"] / 1e9, "structure": desc, "schedule": main["schedule"],
            "factor_step_ms": {name: c[3 * k] / args.steps for k, name in
                               enumerate(["gemm", "potrf", "trsm", "extadd", "qr", "identity", "-",
                                          "fused_cholesky"]) if name != "-"},
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---- the serving stream ------------------------------------------------------
SERVING_POOL = [(2, side) for side in (64, 128, 256, 512, 768, 1024)] + \
               [(3, side) for side in (16, 32, 48, 64, 80, 96)]
SERVING_RHS_POOL = 32   # random right-hand sides kept per matrix; a request takes a window of them


def serving_stream(count, rate, seed):
    """Arrival times, matrix ids, RHS counts and RHS offsets from one MT19937 stream."""
    rng = np.random.RandomState(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    mids = rng.randint(0, len(SERVING_POOL), count)
    nrhs = rng.randint(1, 17, count)
    offs = rng.randint(0, SERVING_RHS_POOL - 16 + 1, count)
    return arrivals, mids, nrhs, offs


def serving_pool(ids, cpu_only=False):
    if cpu_only:
        from oracle import pyoracle as gen
    else:
        import rank_structured_cholesky_gb300 as gen
    probs, rhs = {}, {}
    for m in ids:
        dim, side = SERVING_POOL[m]
        probs[m] = gen.diffusion(dim, side, sigma=1.0, seed=100 + m, nrhs=1)
        rhs[m] = np.random.RandomState(1000 + m).standard_normal((SERVING_RHS_POOL, probs[m].n))
    return probs, rhs


def serve_stream(rs, precision, device, probs, rhs, stream, workers, budget, eps=1e-8, keep=0):
    """Submit the stream in real time, collect every result; returns the measurements."""
    arrivals, mids, nrhs, offs = stream
    srv = rs.Server(workers=workers, hbm_budget_bytes=budget, precision=precision, device=device)
    rids = [None] * len(arrivals)
    results = [None] * len(arrivals)
    ready = threading.Semaphore(0)

    def collect():
        for i in range(len(arrivals)):
            ready.acquire()
            results[i] = srv.wait(rids[i])

    th = threading.Thread(target=collect)
    th.start()
    t0 = time.perf_counter()
    for i in range(len(arrivals)):
        delay = t0 + arrivals[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        m = int(mids[i])
        p = probs[m]
        B = rhs[m][offs[i]:offs[i] + nrhs[i]]
        rids[i] = srv.submit(m, p.colptr, p.rowind, p.vals, B, p.xyz, eps=eps)
        ready.release()
    th.join()
    wall = time.perf_counter() - t0
    stats = srv.stats()
    srv.close()
    lat = np.array([r[3]["latency"] for r in results])
    status = [r[0] for r in results]
    true_res = max(max(q["true_residual"] for q in r[2]) for r in results)
    hits = [r[3]["cache_hit"] for r in results]
    lat_hit = lat[np.array(hits, bool)] if any(hits) else lat
    kept = [results[i][1] for i in range(min(keep, len(results)))]   # solutions of the first requests
    return {"value": len(arrivals) / wall, "rhs_per_s": float(np.sum(nrhs)) / wall, "wall_s": wall, "_kept": kept,
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "p50_ms_cache_hits": 1e3 * float(np.percentile(lat_hit, 50)),
            "p99_ms_cache_hits": 1e3 * float(np.percentile(lat_hit, 99)),
            "failed": int(sum(1 for st in status if st != 0)), "max_true_residual": float(true_res),
            "cache": {k: stats[k] for k in ("hits", "misses", "evictions", "peak_cached_bytes")},
            "h2d_bytes": int(sum(8 * probs[int(m)].n * int(k) for m, k in zip(mids, nrhs))),
            "iterations_mean": float(np.mean([q["iterations"] for r in results for q in r[2]]))}


def serving_cpu_sample(stream, probs, rhs, seconds):
    """The CPU oracle on the stream's requests for the smaller pool matrices
    (factor cached per matrix, as the server does) for about `seconds`."""
    from oracle import pyoracle as po
    small = [i for i in range(len(stream[0])) if probs[int(stream[1][i])].n <= 40000]
    facs, done, t0 = {}, 0, time.perf_counter()
    for i in small:
        m = int(stream[1][i])
        if m not in facs:
            p = probs[m]
            facs[m] = po.OracleFactor(p.colptr, p.rowind, p.vals, p.xyz, dict())
            assert facs[m].factor() == 0
        for j in range(int(stream[2][i])):
            facs[m].pcg(rhs[m][stream[3][i] + j], 1e-8, 10000)
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": done / el, "unit": "requests/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "the first %d requests of the stream whose matrix has n <= 40000 (of %d such), FP64 "
                      "oracle factor cached per matrix + PCG per RHS, threaded BLAS; larger matrices cost more"
                      % (done, len(small))}


def run_serving(args):
    import torch
    import rank_structured_cholesky_gb300 as rs
    rank, world, dist = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    count, rate = args.requests, args.rate
    stream = serving_stream(count, rate, seed=5)
    probs, rhs = serving_pool(sorted(set(int(m) for m in stream[1])))
    budget = args.hbm_budget_gb * 1e9
    prec = 0 if args.precision == "fp64" else 1
    # warm-up: a short stream on the two smallest matrices (CUDA context, module loading)
    warm = (np.arange(args.warmup * 4) * 0.002, np.array([0, 6] * (args.warmup * 2)),
            np.full(args.warmup * 4, 4), np.zeros(args.warmup * 4, int))
    wprobs, wrhs = serving_pool([0, 6])
    serve_stream(rs, prec, local, wprobs, wrhs, warm, args.workers, budget)
    with ClockSampler(local) as clocks:
        main = serve_stream(rs, prec, local, probs, rhs, stream, args.workers, budget, keep=50)
    plain = None
    if args.precision == "mixed" and not args.no_fp64_plain:
        plain = serve_stream(rs, 0, local, probs, rhs, stream, args.workers, budget, keep=50)
        # the mixed results against the FP64 path, request by request (first 50 requests)
        errs = [np.linalg.norm(a - b) / np.linalg.norm(b) for a, b in zip(main["_kept"], plain["_kept"])]
        main["solution_rel_error_vs_fp64"] = {"max": float(max(errs)), "median": float(np.median(errs)),
                                              "requests": len(errs)}
    for d in (main, plain):
        if d:
            d.pop("_kept", None)
    hbm, bf16, src = peaks()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        cpu = serving_cpu_sample(stream, probs, rhs, 20.0)
    if rank == 0:
        line = {
            "metric": "serving: solve requests/s to 1e-8 relative residual", "value": main["value"],
            "unit": "requests/s", "n_gpus": world, "steps": 1, "warmup": args.warmup,
            "ms_per_step": 1e3 * main["wall_s"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == 0 else "f32 factor / f64 pcg", "data": "synthetic",
            "config": {"workload": "c5", "description": CONFIGS["c5"][0], "requests": count, "rate_per_s": rate,
                       "pool": ["%dD side %d (n=%d)" % (d, sd, probs[m].n) for m, (d, sd) in enumerate(SERVING_POOL)
                                if m in probs],
                       "workers": args.workers, "hbm_budget_gb": args.hbm_budget_gb, "precision": args.precision,
                       "l2": "inputs larger than L2 (largest matrices)"},
            "e2e": {"value": main["value"], "unit": "requests/s", "h2d_bytes_per_step": main["h2d_bytes"],
                    "d2h_bytes_per_step": main["h2d_bytes"]},
            "p50_ms": main["p50_ms"], "p99_ms": main["p99_ms"], "serving": main, "plain_fp64": plain,
            "cpu_baseline": cpu, "clocks": clocks.summary(), "peak_source": src,
        }
        print(json.dumps(line), flush=True)
    return 0


def profile_phases(lib, F, ctx, stream, d_b, nrhs, torch):
    """CUDA-event timings of one preconditioner apply and one SpMV, launch counts."""
    out = np.zeros(16)
    st = lib.rschol_profile(F.h, d_b.data_ptr(), out.ctypes.data)
    if st != 0:
        raise RuntimeError("rschol_profile failed: %s" % ctx.last_error())
    return {"factor_ms": out[0], "apply_ms": out[1], "spmv_ms": out[2], "pcg_ms": out[3],
            "apply_bytes": out[4], "spmv_bytes": out[5], "factor_launches": out[6], "pcg_launches": out[7]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--requests", type=int, default=2000, help="c5: requests in the stream")
    ap.add_argument("--rate", type=float, default=200.0,
                    help="c5: mean Poisson arrival rate, requests/s (200 saturates one GB300; a lower rate "
                         "measures latency below saturation)")
    ap.add_argument("--workers", type=int, default=8, help="c5: server worker threads")
    ap.add_argument("--hbm-budget-gb", type=float, default=200.0, help="c5: device bytes for cached factors")
    ap.add_argument("--profile", action="store_true",
                    help="warm up, then run the steps between cudaProfilerStart/Stop (for ncu), no timing line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c5":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
