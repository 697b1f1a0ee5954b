"""Benchmark of the GB300 doubly periodic Stokes mobility operator.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2_dp_n65536] [--precision mixed|fp64]

One step = one Mdot (forces + torques -> linear + angular velocities) of the
named workload with synthetic seeded inputs (default: the open doubly
periodic box with 65,536 particles, 512 x 512 x 128 grid, torques; the
configuration the headline "Mdot particles/s at N=64K" is quoted on).
Prints one JSON line.

ours      : the mixed-precision operator, inputs resident on the device,
            K Mdots between CUDA events (barrier + synchronize on both sides,
            max over ranks); `e2e` is the same metric through the C ABI with
            host arrays (host->device and device->host copies inside the timed
            region); the plain FP64 operator is timed alongside for the
            mixed-vs-FP64 part of the metric; `roofline` is the dominant
            stage from CUDA events over K timed Mdots.
reference : the reference CPU path as restated by the oracle (the reference's
            own compiled CPU code cannot be built on this host: its sources
            are not shipped here), whole Mdots of the same workload on every
            host core (oracle/cpu_parallel.py: worker processes dividing the
            spreading by grid-column groups, the solve by wavenumber blocks
            and the interpolation by particles, transforms on scipy.fft's
            threads), W untimed and K timed, nothing sampled or scaled; the
            same measurement (one warm-up, one timed Mdot) is this arm's
            `cpu_baseline`.
Under torchrun (N > 1) every rank runs an independent replica (one system
does not shard: replicas only); value aggregates over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mdot particles/s at N=64K, mixed vs FP64 at rel err<=1e-5; bwd/fwd time ratio"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap,power.draw")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.file is None:
            return None
        try:
            rows = [l.strip().split(", ") for l in open(self.file.name) if l.strip()]
            os.unlink(self.file.name)
        except Exception:
            return None
        sm = [float(r[0]) for r in rows if len(r) >= 7 and r[0].replace('.', '').isdigit()]
        mx = [float(r[1]) for r in rows if len(r) >= 7 and r[1].replace('.', '').isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 7 for i in range(4)
                          if r[2 + i].strip().lower() == "active"})
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def algorithmic_bytes(stage, w, prec, arith=None):
    """Bytes a stage must move at minimum for one Mdot: the grid (3 nx ny nz
    values) and / or the spectrum (3 nz ny (nx/2+1) complex values) once in
    and once out, the per-wavenumber factors of the solve, and the particle
    data.  `arith` "double-float" counts the double-float solve's factors
    (kappa and A^-1 B per row, 2 nz float2, and 64 B of Ginv, K^2, H^2 K
    scalars per wavenumber); otherwise the FP64 solve's 6 nz + 4 FP64 values."""
    s = 4 if prec == "mixed" else 8
    nxh = w.nx // 2 + 1
    nk = w.ny * nxh
    grid = 3 * w.nx * w.ny * w.nz * s
    spec = 3 * nk * w.nz * 2 * s
    if stage == "solve" and w.domType == "TP":
        # triply periodic: the spectrum in and out (wavenumber tables are cached)
        return 2 * spec
    if stage == "solve" and arith == "double-float":
        return 2 * spec + nk * (2 * w.nz * 8 + 64)
    if stage == "solve":
        # spectrum in and out, per-wavenumber factors (6 nz + 4 FP64 values)
        return 2 * spec + nk * (6 * w.nz + 4) * 8
    if stage in ("ztrans_fwd", "ztrans_inv"):
        return 2 * spec
    if stage in ("fft_fwd", "fft_inv"):
        return grid + spec
    if stage == "spread":
        return grid + w.N * (6 if w.has_torque else 3) * s
    if stage == "interp":
        return grid + w.N * (6 if w.has_torque else 3) * s
    return None


def max_over_ranks(x, world, device):
    """The maximum of a per-rank scalar over the job's ranks (the replicas
    time the same workload independently; the job's time is the slowest)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_particles, steps, seconds, world):
    """Whole-job particles/s: every rank runs its own replica of the workload
    (no data-path collective), so the units are world x N x steps over the
    slowest rank's time."""
    return world * n_particles * steps / seconds


def run_ours(args, rank, world):
    import torch
    import ctypes
    from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W, _lib
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = W.by_name(args.workload)
    X, F, T = W.make_inputs(w)
    prec = args.precision
    dt = torch.float32 if prec == "mixed" else torch.float64

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    prm = StokesParams.from_workload(w, prec)
    if args.solve != "default":
        prm = StokesParams(**{**prm.as_dict(), "solve": args.solve})
    op = DPStokes(prm, w.N, device=dev)
    op.set_positions(torch.tensor(X, device=dev))
    Fd = torch.tensor(F, dtype=dt, device=dev)
    Td = torch.tensor(T, dtype=dt, device=dev) if T is not None else None
    V = torch.empty_like(Fd)
    Wd = torch.empty_like(Fd) if w.has_torque else None
    for _ in range(args.warmup):
        op.mdot(Fd, Td, out=(V, Wd))
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as cs:
        barrier()
        e0.record()
        for _ in range(args.steps):
            op.mdot(Fd, Td, out=(V, Wd))
        e1.record()
        barrier()
    ms = e0.elapsed_time(e1)
    clocks = cs.summary()
    ms = max_over_ranks(ms, world, dev)
    ms_step = ms / args.steps
    value = replica_value(w.N, args.steps, ms / 1e3, world)

    # per-stage device times (CUDA events on the operator's stream)
    stage_runs = []
    for _ in range(max(3, min(args.steps, 10))):
        _, _, st = op.mdot_timed(Fd, Td)
        stage_runs.append(st)
    stages = {k: statistics.median([s[k] for s in stage_runs]) for k in stage_runs[0]}
    info = op.info()

    # a position update (locate, stencils, ghost layers, tile order; one host
    # synchronisation for the error flags), wall clock per call
    Xd = torch.tensor(X, device=dev)
    for _ in range(2):
        op.set_positions(Xd)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        op.set_positions(Xd)
    torch.cuda.synchronize()
    set_positions_ms = (time.perf_counter() - t0) * 1e3 / 10

    # end to end through the C ABI with pinned host arrays
    L = _lib.lib()
    Fh = torch.tensor(F, dtype=dt).pin_memory()
    Th = torch.tensor(T, dtype=dt).pin_memory() if T is not None else None
    Vh = torch.empty_like(Fh).pin_memory()
    Wh = torch.empty_like(Fh).pin_memory() if w.has_torque else None
    code = _lib.F32 if dt == torch.float32 else _lib.F64
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None else 0)  # noqa: E731

    def e2e_step():
        _lib.check(L.dpst_mdot_host(op._h, ptr(Fh), ptr(Th), ptr(Vh), ptr(Wh), code, stream))

    for _ in range(2):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    nbytes = Fh.numel() * Fh.element_size()

    # the allocation-free entry point on device arrays (static solve scratch,
    # FP64-arithmetic solve on as many CTAs as the static array holds)
    def noalloc_step():
        _lib.check(L.dpst_mdot_noalloc(op._h, ptr(Fd), ptr(Td), ptr(V), ptr(Wd), code, stream))

    for _ in range(2):
        noalloc_step()
    barrier()
    k_na = max(3, min(args.steps, 10))
    e0.record()
    for _ in range(k_na):
        noalloc_step()
    e1.record()
    barrier()
    noalloc_ms = e0.elapsed_time(e1) / k_na
    e2e = {"value": replica_value(w.N, args.steps, e2e_s, world), "unit": "particles/s",
           "h2d_bytes_per_step": nbytes * (2 if T is not None else 1),
           "d2h_bytes_per_step": nbytes * (2 if w.has_torque else 1)}

    # the plain FP64 operator on the same inputs: speed and error of mixed
    extra = {}
    if prec == "mixed" and not args.skip_fp64:
        op64 = DPStokes(StokesParams.from_workload(w, "fp64"), w.N, device=dev)
        op64.set_positions(torch.tensor(X, device=dev))
        F64 = torch.tensor(F, device=dev)
        T64 = torch.tensor(T, device=dev) if T is not None else None
        V64, W64 = op64.mdot(F64, T64)
        barrier()
        k64 = max(2, args.steps // 5)
        e0.record()
        for _ in range(k64):
            op64.mdot(F64, T64)
        e1.record()
        barrier()
        ms64 = e0.elapsed_time(e1) / k64
        V32, W32 = op.mdot(Fd, Td)
        torch.cuda.synchronize()
        rel = lambda a, b: float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))  # noqa: E731
        extra = {"fp64_particles_per_s": w.N / (ms64 / 1e3), "fp64_ms_per_step": ms64,
                 "speedup_vs_fp64": ms64 / ms_step, "rel_err_V_vs_fp64": rel(V32, V64)}
        if W64 is not None:
            extra["rel_err_W_vs_fp64"] = rel(W32, W64)
        op64.close()

    # roofline of the dominant stage
    peaks, peak_kind = load_peaks()
    stage_names = [k for k in stages if k != "total"]
    dom = max(stage_names, key=lambda k: stages[k])
    arith = {1: "fp64", 2: "double-float"}.get(info.get("solve_arith"), "n/a")
    ab = algorithmic_bytes(dom, w, prec, arith)
    achieved = ab / (stages[dom] * 1e-3) / 1e9 if ab else None
    roof = {"bound": "hbm", "stage": dom, "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": None, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}
    # every stage against HBM from the same CUDA-event stage times
    roof["stages"] = {}
    for k in stage_names:
        b = algorithmic_bytes(k, w, prec, arith)
        if b and stages[k] > 0:
            gbs = b / (stages[k] * 1e-3) / 1e9
            roof["stages"][k] = {"ms": round(stages[k], 4), "algorithmic_bytes": b,
                                 "achieved_gbs": round(gbs, 1), "frac": round(gbs / peaks["hbm_gbs"], 4)}
    # the z transform as a dense contraction: 2 nz^2 flops per real column (3 x 2 nk columns) per
    # product, three TF32 products (split TF32) on the tensor pipe; TF32 dense rate taken as half
    # the measured BF16 rate
    if w.domType != "TP" and info.get("ztransform") in (1, 3) and stages.get("ztrans_fwd", 0) > 0:
        nk = w.ny * (w.nx // 2 + 1)
        flops = 3 * 2.0 * w.nz * w.nz * 3 * 2 * nk
        tf32_peak = peaks["bf16_tflops"] / 2.0
        roof["ztransform_tensor"] = {
            "tf32_flops_per_transform": flops,
            "achieved_tflops_fwd": flops / (stages["ztrans_fwd"] * 1e-3) / 1e12,
            "achieved_tflops_inv": flops / (stages["ztrans_inv"] * 1e-3) / 1e12,
            "peak_tflops": tf32_peak, "peak_source": peak_kind + " bf16_tflops / 2 (TF32 dense)",
            "frac_fwd": flops / (stages["ztrans_fwd"] * 1e-3) / 1e12 / tf32_peak}
    znames = {0: "SIMT folded", 1: "tcgen05 split-TF32", 2: "double-float SIMT",
              3: "tcgen05 split-TF32, TMA-fed"}
    roof["ztransform_kernel"] = znames.get(info.get("ztransform"), "SIMT folded")
    roof["ztransform_inverse_kernel"] = znames.get(info.get("ztransform_inverse"), "SIMT folded")
    if info.get("ztransform_tma_ms") and info["ztransform_tma_ms"][0] > 0:
        roof["ztransform_creation_ms"] = {
            "forward": {"simt": round(float(info["ztransform_ms"][0]), 4),
                        "tcgen05": round(float(info["ztransform_ms"][1]), 4),
                        "tcgen05_tma": round(float(info["ztransform_tma_ms"][0]), 4)},
            "inverse": {"simt": round(float(info["ztransform_inverse_ms"][0]), 4),
                        "tcgen05": round(float(info["ztransform_inverse_ms"][1]), 4),
                        "tcgen05_tma": round(float(info["ztransform_tma_ms"][1]), 4)},
            "tma_variant": list(info["ztransform_tma_variant"]),
            "tma_variants_ms": [round(float(x), 4) for x in info["ztransform_tma_variant_ms"]]}
    if dom == "solve" and arith == "double-float":
        # the double-float solve is issue bound (FP32 FMA chains of the
        # compensated sweeps): its DRAM traffic is measured by ncu, and the
        # issue rate is its warp instructions over the SMs' issue slots
        roof["note"] = ("per-wavenumber double-float BVP: issue bound (FP32 FMA pipe); HBM fraction "
                        "is of its algorithmic bytes; issue gives warp instructions per issue slot")
        nk_solve = w.ny * (w.nx // 2 + 1)
        if w.domType == "DP" and w.nz == 128:
            # ncu launch list of the c2 Mdot (512^2 x 128 open box, 131,584 wavenumbers):
            # k_bvp_df variant 3 read 1065.8 MB and wrote 615.5 MB per launch
            roof["traffic"] = (1065.8e6 + 615.5e6) / 131584 * nk_solve
            roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_bvp_df "
                                      "(variant 3) on c2_dp_n65536, per launch, scaled by wavenumbers "
                                      "(profiles/launches_c2_dp_n65536_mixed.md)")
            # 636 M warp instructions for the 74,112 wavenumbers of c2_dp_n65536@384
            # (ncu smsp__inst_executed.sum; profiles/k_bvp_df_c2_at384_dp_n36864_mixed.md)
            nsm = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = clocks.get("sm_mhz") or 2070.0
            instr = 636e6 / 74112 * nk_solve
            rate = instr / (stages["solve"] * 1e-3)
            peak = nsm * 4 * mhz * 1e6
            roof["issue"] = {"warp_instructions": instr, "achieved_per_s": rate, "peak_per_s": peak,
                             "frac": rate / peak, "sm_mhz": mhz, "sms": nsm}
    elif dom == "solve":
        # FP64-pipe bound: report the FP64 arithmetic rate against the GB300 FP64 peak
        roof["note"] = ("per-wavenumber FP64 BVP: FP64-pipe bound; HBM fraction shown is of "
                        "its algorithmic bytes; fp64_pipe gives its FP64 issue rate")
        if w.domType == "DP" and w.nz == 128:
            # DRAM bytes of the hybrid solve per wavenumber from the ncu capture of
            # k_bvp_hybrid on c2_dp_n65536@384 (same geometry and nz: 3.42 GB read +
            # 1.32 GB written for 74,112 wavenumbers), scaled by this grid's wavenumbers
            nk_solve = w.ny * (w.nx // 2 + 1)
            roof["traffic"] = (3.42e9 + 1.32e9) / 74112 * nk_solve
            roof["traffic_source"] = ("ncu k_bvp_hybrid on c2_dp_n65536@384, scaled by wavenumbers "
                                      "(profiles/k_bvp_hybrid_c2_at384_dp_n36864_mixed.md)")
        if w.domType != "TP":
            # ~46 FP64 instructions per row per lane (2 lanes x nz rows per wavenumber;
            # ncu's FP64 instruction count of the solve), at 2 FP64 lane-operations
            # per clock per SM
            nsm = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = clocks.get("sm_mhz") or 2070.0
            instr = (w.ny * (w.nx // 2 + 1) - 1) * 2 * w.nz * 46
            rate = instr / (stages["solve"] * 1e-3)
            peak = nsm * 2 * mhz * 1e6
            roof["fp64_pipe"] = {"lane_instructions": instr, "achieved_per_s": rate, "peak_per_s": peak,
                                 "frac": rate / peak, "sm_mhz": mhz, "sms": nsm}
    extra["xy_transform"] = {"form": {0: "cuFFT", 1: "own, two passes", 2: "own, one launch",
                                      3: "own double-float, two passes",
                                      4: "own, one launch of 8-CTA clusters"}.get(
        info.get("xy_transform"), "n/a"), "pair_ms_two_pass_one_launch": [round(float(x), 4) for x in
                                                                        info.get("xy_ms", [])],
        "pair_ms_cluster": round(float(info.get("xy_cluster_ms", 0.0)), 4)}
    extra["set_positions_ms"] = set_positions_ms
    extra["noalloc_ms_per_step"] = noalloc_ms
    extra["solve_kernel"] = {"arith": arith,
                             "variant": info.get("solve_variant"),
                             "variant_ms": [round(float(x), 4) for x in info.get("solve_ms", [])]}
    return dict(value=value, ms_step=ms_step, e2e=e2e, stages=stages, info=info, extra=extra,
                roofline=roof, clocks=clocks, w=w)


def run_backward(args, dev, precision="fp64"):
    """Forward and backward (dl/dF and dl/dX of l = <g, M(X) F>) of the
    differentiation configuration: bottom wall, N = 8192, 192^2 x 64, forces
    only.  Returns device milliseconds per call of each and their ratio."""
    import torch
    from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W
    w = W.C3
    X, F, _ = W.make_inputs(w)
    dt = torch.float64 if precision == "fp64" else torch.float32
    g = np.random.default_rng(12).standard_normal((w.N, 3))
    op = DPStokes(StokesParams.from_workload(w, precision), w.N, device=dev)
    op.set_positions(torch.tensor(X, device=dev))
    Fd = torch.tensor(F, dtype=dt, device=dev)
    gd = torch.tensor(g, dtype=dt, device=dev)
    V = torch.empty_like(Fd)
    k = max(3, min(args.steps, 20))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    fwd = timed(lambda: op.mdot(Fd, None, out=(V, None)))

    def step():
        # a training step: the forward, then the backward on the forward's
        # velocity grid (dpst_mdot_backward_saved)
        op.mdot(Fd, None, out=(V, None))
        op.mdot_backward(Fd, None, gd, need_F=True, need_X=True, forward_serial=op.forward_serial())

    pair = timed(step)
    reused = op.last_backward_reused
    bwd_re = timed(lambda: op.mdot_backward(Fd, None, gd, need_F=True, need_X=True))
    op.close()
    bwd = pair - fwd
    return {"workload": w.name, "precision": precision, "grads": ["F", "X"], "calls": k,
            "fwd_ms": fwd, "bwd_ms": bwd, "bwd_fwd_ratio": bwd / fwd, "fwd_bwd_pair_ms": pair,
            "forward_grid_reused": reused, "bwd_recompute_ms": bwd_re, "bwd_recompute_fwd_ratio": bwd_re / fwd,
            "note": "bwd_ms = (forward + backward on the forward's velocity grid) - forward; "
                    "bwd_recompute_ms: a backward that recomputes the forward's spread and velocity grid"}


def run_batched(args, dev):
    """The batched bottom-wall configuration: 256 systems, N_i log-uniform in
    [64, 4096], L_i ~ U[32, 128], mixed precision.  One batched Mdot (a
    captured graph over all systems) against a loop of the 256 single-system
    operators on the same inputs; device milliseconds per pass over all
    systems."""
    import torch
    from doublyperiodicstokes_gb300 import DPStokes, DPStokesBatch, StokesParams, workloads as W
    ws = W.batched_c4()
    prm = [StokesParams.from_workload(w, "mixed") for w in ws]
    ins = [W.make_inputs(w) for w in ws]
    X = torch.tensor(np.concatenate([a[0] for a in ins]), device=dev)
    F = torch.tensor(np.concatenate([a[1] for a in ins]), dtype=torch.float32, device=dev)
    b = DPStokesBatch(prm, [w.N for w in ws], device=dev)
    b.set_positions(X)
    V = torch.empty_like(F)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    k = max(3, min(args.steps, 10))

    def timed(fn, reps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    batched = timed(lambda: b.mdot(F, None, out=(V, None)), k)
    info = b.info()
    b.close()
    ops, Fs = [], []
    for w, p, a in zip(ws, prm, ins):
        op = DPStokes(p, w.N, device=dev)
        op.set_positions(torch.tensor(a[0], device=dev))
        ops.append(op)
        Fs.append(torch.tensor(a[1], dtype=torch.float32, device=dev))
    Vs = [torch.empty_like(f) for f in Fs]

    def loop():
        for op, f, v in zip(ops, Fs, Vs):
            op.mdot(f, None, out=(v, None))

    looped = timed(loop, max(2, k // 3))
    for op in ops:
        op.close()
    n = sum(w.N for w in ws)
    return {"workload": "c4_dpbw_256sys", "systems": len(ws), "particles": n,
            "size_classes": info["n_size_classes"], "modes": info["n_modes"],
            "batched_ms": batched, "loop_ms": looped, "speedup_vs_loop": looped / batched,
            "batched_particles_per_s": n / (batched / 1e3), "loop_particles_per_s": n / (looped / 1e3),
            "kernels_per_batched_mdot": info["kernels_per_mdot"], "fft_plans": info["fft_plans"],
            "ztransform": {1: "tcgen05", 3: "tcgen05, TMA-fed", 0: "SIMT"}.get(info["ztransform"]),
            "ztransform_inverse": {1: "tcgen05", 3: "tcgen05, TMA-fed", 0: "SIMT"}.get(info["ztransform_inverse"]),
            "ztransform_ms_simt_tcgen05": [round(float(x), 3) for x in info["ztransform_ms"]],
            "ztransform_inverse_ms_simt_tcgen05": [round(float(x), 3) for x in info["ztransform_inverse_ms"]],
            "ztransform_tma_ms_fwd_inv": [round(float(x), 3) for x in info["ztransform_tma_ms"]],
            "precision": "mixed", "note": "one CUDA graph launch per batched Mdot"}


def run_multi_rhs(args, dev):
    """Multi-RHS Mdot (dpst_mdot_multi): K columns at the same positions against
    K single Mdots on the same handle; c0 (FP64, K = 16, the mobility-matrix
    use) and c2 (mixed, K = 4).  Device milliseconds per column."""
    import torch
    from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = max(3, min(args.steps, 10))

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    out = []
    for w, precision, K in ((W.C0, "fp64", 16), (W.C2, "mixed", 4)):
        dt = torch.float64 if precision == "fp64" else torch.float32
        X, _, _ = W.make_inputs(w)
        rng = np.random.default_rng(3)
        F = torch.tensor(rng.standard_normal((K, w.N, 3)), dtype=dt, device=dev)
        T = torch.tensor(rng.standard_normal((K, w.N, 3)), dtype=dt, device=dev) if w.has_torque else None
        op = DPStokes(StokesParams.from_workload(w, precision), w.N, device=dev)
        op.set_positions(torch.tensor(X, device=dev))
        V = torch.empty_like(F)
        Wt = torch.empty_like(F) if w.has_torque else None
        multi = timed(lambda: op.mdot_multi(F, T, out=(V, Wt)))

        def loop():
            for k in range(K):
                op.mdot(F[k], T[k] if T is not None else None,
                        out=(V[k], Wt[k] if Wt is not None else None))

        single = timed(loop)
        op.close()
        out.append({"workload": w.name, "precision": precision, "columns": K,
                    "multi_ms_per_column": multi / K, "single_ms_per_column": single / K,
                    "speedup": single / multi,
                    "multi_particle_columns_per_s": w.N * K / (multi / 1e3)})
    return out


def run_periodic(args, dev):
    """Triply periodic Mdot on t1_tp_n65536 (512 x 512 x 64, N = 65,536,
    torques): mixed and FP64 operators, device milliseconds per Mdot and per
    backward (dl/dF, dl/dT, dl/dX), the CUDA-event stage split with each
    stage's HBM fraction, mixed vs FP64."""
    import torch
    from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W
    w = W.T1
    X, F, T = W.make_inputs(w)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = max(3, min(args.steps, 10))
    peaks, _ = load_peaks()
    out = {"workload": w.name, "grid": [w.nx, w.ny, w.nz], "N": w.N}
    res = {}
    for precision in ("mixed", "fp64"):
        dt = torch.float32 if precision == "mixed" else torch.float64
        op = DPStokes(StokesParams.from_workload(w, precision), w.N, device=dev)
        op.set_positions(torch.tensor(X, device=dev))
        Fd = torch.tensor(F, dtype=dt, device=dev)
        Td = torch.tensor(T, dtype=dt, device=dev)
        V = torch.empty_like(Fd)
        Wd = torch.empty_like(Fd)
        for _ in range(max(3, args.warmup)):
            op.mdot(Fd, Td, out=(V, Wd))
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            op.mdot(Fd, Td, out=(V, Wd))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        runs = [op.mdot_timed(Fd, Td)[2] for _ in range(reps)]
        st = {k: statistics.median([r[k] for r in runs]) for k in runs[0]}
        st = {k: v for k, v in st.items() if not k.startswith("ztrans")}
        roof = {}
        for k, v in st.items():
            b = algorithmic_bytes(k, w, precision)
            if b and v > 0:
                gbs = b / (v * 1e-3) / 1e9
                roof[k] = {"achieved_gbs": round(gbs, 1), "frac": round(gbs / peaks["hbm_gbs"], 4)}
        res[precision] = (V.double().clone(), Wd.double().clone())
        # backward: dl/dF, dl/dT, dl/dX of l = <gV, V> + <gW, W>
        gVd = torch.tensor(np.random.default_rng(12).standard_normal(F.shape), dtype=dt, device=dev)
        gWd = torch.tensor(np.random.default_rng(13).standard_normal(F.shape), dtype=dt, device=dev)
        def timed_loop(fn):
            for _ in range(max(3, args.warmup)):
                fn()
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        def step():
            # forward, then the backward on the forward's velocity grid
            op.mdot(Fd, Td, out=(V, Wd))
            op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_T=True, need_X=True,
                             forward_serial=op.forward_serial())

        pair = timed_loop(step)
        reused = op.last_backward_reused
        bre = timed_loop(lambda: op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_T=True, need_X=True))
        bms = pair - ms
        out[precision] = {"ms_per_mdot": ms, "particles_per_s": w.N / (ms / 1e3),
                          "stages_ms": {k: round(v, 4) for k, v in st.items()}, "stage_hbm": roof,
                          "kernels_per_mdot": op.info()["kernels_per_mdot"],
                          "backward_ms": bms, "bwd_fwd_ratio": bms / ms, "backward_grads": ["F", "T", "X"],
                          "fwd_bwd_pair_ms": pair, "forward_grid_reused": reused,
                          "backward_recompute_ms": bre, "bwd_recompute_fwd_ratio": bre / ms}
        op.close()
    rel = lambda a, b: float(torch.linalg.norm(a - b) / torch.linalg.norm(b))  # noqa: E731
    out["rel_err_V_mixed_vs_fp64"] = rel(res["mixed"][0], res["fp64"][0])
    out["rel_err_W_mixed_vs_fp64"] = rel(res["mixed"][1], res["fp64"][1])
    out["speedup_mixed_vs_fp64"] = out["fp64"]["ms_per_mdot"] / out["mixed"]["ms_per_mdot"]
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(w)
    return out


def run_regkernel(args, dev):
    """The regular-kernel torque coupling (the reference's useRegKernel) on c2
    and t1, mixed: device milliseconds per Mdot and the CUDA-event stage split,
    beside the derivative-kernel coupling on the same inputs."""
    import dataclasses
    import torch
    from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = max(3, min(args.steps, 10))
    out = []
    for base in (W.C2, W.T1):
        X, F, T = W.make_inputs(base)
        row = {"workload": base.name, "precision": "mixed"}
        for reg in (False, True):
            w = dataclasses.replace(base, reg_kernel=reg)
            op = DPStokes(StokesParams.from_workload(w, "mixed"), w.N, device=dev)
            op.set_positions(torch.tensor(X, device=dev))
            Fd = torch.tensor(F, dtype=torch.float32, device=dev)
            Td = torch.tensor(T, dtype=torch.float32, device=dev)
            V, Wd = torch.empty_like(Fd), torch.empty_like(Fd)
            for _ in range(max(3, args.warmup)):
                op.mdot(Fd, Td, out=(V, Wd))
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                op.mdot(Fd, Td, out=(V, Wd))
            e1.record()
            torch.cuda.synchronize()
            key = "reg_kernel" if reg else "deriv_kernel"
            row[key + "_ms"] = e0.elapsed_time(e1) / reps
            if reg:
                runs = [op.mdot_timed(Fd, Td)[2] for _ in range(reps)]
                row["reg_kernel_stages_ms"] = {k: round(statistics.median([r[k] for r in runs]), 4)
                                               for k in runs[0]}
                row["reg_kernel_particles_per_s"] = w.N / (row[key + "_ms"] / 1e3)
            op.close()
        out.append(row)
    return out


def cpu_baseline(w, steps=1, warmup=1):
    """Whole Mdots of the oracle (the reference CPU path restated) on every
    host core this process may use (oracle/cpu_parallel.py): set-up untimed,
    `warmup` untimed Mdots, then `steps` timed ones, nothing sampled.  The
    triply periodic mode, which that module does not cover, falls back to the
    single-threaded sample of oracle/cpu_sample.py, labelled as such."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import dpstokes_oracle as O
    from doublyperiodicstokes_gb300 import workloads as W
    X, F, T = W.make_inputs(w)
    p = O.Params(**w.oracle_params())
    if w.domType == "TP" or w.reg_kernel:
        import cpu_sample
        tot, stages, sample = cpu_sample.sample_mdot_seconds(p, X, F, T)
        return {"value": w.N / tot, "unit": "particles/s", "cores": 1, "kind": "port",
                "sample": "extrapolated: " + sample, "seconds_per_mdot": tot, "measured": False,
                "stage_seconds": {k: round(v, 3) for k, v in stages.items()}}
    import cpu_parallel
    t0 = time.perf_counter()
    pm = cpu_parallel.ParallelMdot(p, X)
    setup = time.perf_counter() - t0
    try:
        for _ in range(warmup):
            pm.mdot(F, T)
        times, stage_runs = [], []
        for _ in range(steps):
            t0 = time.perf_counter()
            pm.mdot(F, T)
            times.append(time.perf_counter() - t0)
            stage_runs.append(dict(pm.stage_seconds))
    finally:
        pm.close()
    mean = sum(times) / len(times)
    stages = {k: round(statistics.median([r[k] for r in stage_runs]), 3) for k in stage_runs[0]}
    return {"value": w.N / mean, "unit": "particles/s", "cores": pm.workers, "kind": "port",
            "sample": ("whole Mdots of %s (no sampling, no scaling): %d timed after %d untimed, mean; "
                       "numpy oracle on %d worker processes (spreading by grid-column groups, solve by "
                       "wavenumber blocks, interpolation by particles), transforms on %d scipy.fft threads"
                       % (w.name, steps, warmup, pm.workers, pm.workers)),
            "seconds_per_mdot": mean, "seconds_min": min(times), "seconds_max": max(times),
            "measured": True, "setup_seconds": round(setup, 2), "stage_seconds": stages}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2_dp_n65536")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solve", default="default", choices=["default", "fp64", "df64"],
                    help="arithmetic of the per-wavenumber solve of the timed operator")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-backward", action="store_true")
    ap.add_argument("--only-backward", action="store_true",
                    help="time only the backward pass of the differentiation configuration")
    ap.add_argument("--only-backward-mixed", action="store_true",
                    help="time only the mixed operator's backward pass of the differentiation configuration")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--only-batched", action="store_true",
                    help="time only the batched configuration (256 systems)")
    ap.add_argument("--skip-periodic", action="store_true")
    ap.add_argument("--only-periodic", action="store_true",
                    help="time only the triply periodic Mdot (t1_tp_n65536)")
    ap.add_argument("--skip-regkernel", action="store_true")
    ap.add_argument("--only-regkernel", action="store_true",
                    help="time only the regular-kernel torque coupling (c2, t1)")
    ap.add_argument("--skip-multi", action="store_true")
    ap.add_argument("--only-multi", action="store_true",
                    help="time only the multi-RHS Mdot (c0 K = 16, c2 K = 4)")
    args = ap.parse_args()
    if args.only_regkernel:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"reg_kernel": run_regkernel(args, dev)}), flush=True)
        return
    if args.only_periodic:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"periodic": run_periodic(args, dev)}), flush=True)
        return
    if args.only_multi:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"multi_rhs": run_multi_rhs(args, dev)}), flush=True)
        return
    if args.only_batched:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"batched": run_batched(args, dev)}), flush=True)
        return
    if args.only_backward_mixed:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"backward_mixed": run_backward(args, dev, "mixed")}), flush=True)
        return
    if args.only_backward:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"backward": run_backward(args, dev),
                          "backward_mixed": run_backward(args, dev, "mixed")}), flush=True)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    from doublyperiodicstokes_gb300 import workloads as W
    w = W.by_name(args.workload)
    config = {"workload": w.name, "domain": w.domType, "N": w.N, "grid": [w.nx, w.ny, w.nz],
              "box": [w.Lx, w.Ly, w.Lz], "torques": w.has_torque, "kernel_w": w.wm,
              "precision": args.precision, "l2": "inputs larger than L2 (grid > 129 MB)",
              "parallelism": "replicas x%d" % args.gpus}
    if args.impl == "reference":
        if rank != 0:
            return
        t0 = time.time()
        cb = cpu_baseline(w, steps=args.steps, warmup=args.warmup)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "particles/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * cb["seconds_per_mdot"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config, "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "particles/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "wall_s": time.time() - t0}
        print(json.dumps(line), flush=True)
        return
    r = run_ours(args, rank, world)
    if rank != 0:
        return
    info = r["info"]
    line = {"metric": METRIC, "value": r["value"], "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": config, "e2e": r["e2e"],
            "gpu_launches": info["kernels_per_mdot"] * args.steps,
            "roofline": r["roofline"], "clocks": r["clocks"],
            "stages_ms": {k: round(v, 4) for k, v in r["stages"].items()},
            "bwd_fwd_ratio": None}
    line.update(r["extra"])
    if not args.skip_backward:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        bw = run_backward(args, dev)
        line["backward"] = bw
        line["bwd_fwd_ratio"] = bw["bwd_fwd_ratio"]
        if args.precision == "mixed":
            line["backward_mixed"] = run_backward(args, dev, "mixed")
    if not args.skip_batched:
        import torch
        line["batched"] = run_batched(args, torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))))
    if not args.skip_multi:
        import torch
        line["multi_rhs"] = run_multi_rhs(args, torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))))
    if not args.skip_regkernel:
        import torch
        line["reg_kernel"] = run_regkernel(args, torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))))
    if not args.skip_periodic:
        import torch
        line["periodic"] = run_periodic(args, torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))))
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(r["w"])
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
