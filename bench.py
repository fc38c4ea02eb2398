"""Benchmark: Richardson-Lucy (ISRA) iterations per second on a 1005 x 1005 x 31
volume (Nnum 15, 67 x 67 lenslets, PSF 345 x 345 x 15 x 15 x 31), one GPU.

A step is one ISRA iteration (deconvRL.m:46-87): one forward projection, one
back projection and the fused multiplicative update, computed by libsid with
the method chosen by --method (default: the mixed-precision spectral form,
forward tap spectra stored as 16-bit block floating point, back projection
tap spectra as 24-bit floats with the weakly observed voxels recomputed from
the FP32 taps, FP32 arithmetic).  Inputs are seeded synthetic data with the
shapes of the benchmark configuration.

Prints ONE JSON line (rank 0).  --impl reference times the CPU restatement of
the reference's projection (the FP32 lenslet-sparse loop of oracle/sid_oracle.c,
OpenMP over all host cores) on a bounded column sample, extrapolated to whole
iterations.  Multi-GPU runs (torchrun) are independent replicas: the path has
no exchange step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RL iter/s (1005^2x31)"
UNIT = "iter/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="sid", choices=["sid", "reference"])
    ap.add_argument("--method", default="spectral_mixed",
                    choices=["direct", "spectral_f32", "spectral_i16", "spectral_mixed", "spectral_mixed_f32"])
    ap.add_argument("--compare", default="direct,spectral_f32",
                    help="other methods timed after the main region (comma list, '' for none)")
    ap.add_argument("--compare-steps", type=int, default=3)
    ap.add_argument("--config", default="1005x1005x31", choices=["225x225x11", "1005x1005x31"])
    ap.add_argument("--depths", type=int, default=0,
                    help="keep only the first Z depth planes (a smaller case of the same lateral geometry, for "
                         "profiling captures; the line then names the reduced workload)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-nnls", action="store_true", help="skip the library + temporal NNLS measurement")
    ap.add_argument("--library-only", action="store_true",
                    help="time only the library generation (--nnls-neurons neurons) and print its numbers")
    ap.add_argument("--nnls-frames", type=int, default=3000)
    ap.add_argument("--nnls-neurons", type=int, default=800)
    ap.add_argument("--no-demix", action="store_true", help="skip the demixing-loop measurement")
    ap.add_argument("--batch-volumes", type=int, default=64,
                    help="components deconvolved side by side in the batched measurement (0 skips it)")
    ap.add_argument("--demix-neurons", type=int, default=1500)
    ap.add_argument("--demix-frames", type=int, default=5000)
    ap.add_argument("--demix-iters", type=int, default=5)
    ap.add_argument("--nnls-fp64-frames", type=int, default=192,
                    help="frames of the temporal NNLS solved again in FP64 (oracle) for the accuracy fields")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_throughput(ms, steps, world, device):
    """Whole-job throughput of `world` independent replicas (one per GPU, no
    exchange step): the slowest rank's time (all-reduce MAX over the process
    group) and world * steps iterations in that time."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps / (ms / 1e3)


def workload_name(X, Y, Z, N, M):
    """The workload string both arms print (the same ISRA step on the same data)."""
    return f"ISRA iteration on {X}x{Y}x{Z}, Nnum {N}, PSF {M}^2x{N}^2x{Z}"


def workload(config, depths=0):
    import numpy as np
    from sid_gb300 import synthetic
    H, V = synthetic.config_inputs(config)
    if depths and depths < H.shape[4]:
        H = np.asfortranarray(H[..., :depths])
        V = np.asfortranarray(V[..., :depths])
    return H, V


def cpu_sample(H, V, seconds, nthreads=0):
    """Time the FP32 lenslet-sparse forward projection of oracle/ on a growing
    number of sensor columns until `seconds` of work; returns (seconds per
    projection extrapolated to all columns, columns timed)."""
    from oracle import oracle
    Y = V.shape[1]
    cols, spent = 0, 0.0
    step = 1
    while spent < seconds and cols < Y:
        n = min(step, Y - cols)
        t0 = time.perf_counter()
        oracle.baseline_forward_f32(H, V, cols, cols + n, nthreads)
        spent += time.perf_counter() - t0
        cols += n
        step = min(step * 2, 64)
    return spent / cols * Y, cols, spent


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def library_timing(P_proj, K):
    """Library generation for K anisotropic Gaussian neurons in the projector's
    volume (generate_LFM_library_GPU.m:63-109), timed through the FP32 lenslet
    taps (sid_library) and the tensor-core windows (sid_library_spectral).
    Returns (A (P x K, the FP32 taps' rows, unnormalised), timings)."""
    import ctypes

    import numpy as np
    import torch

    import sid_gb300 as s
    from sid_gb300 import _lib, synthetic
    X, Y, Z = P_proj.X, P_proj.Y, P_proj.Z
    P = X * Y
    vol, centers = synthetic.neuron_volume(X, Y, Z, K)
    neur_id = np.ones((K, 1), dtype=bool)
    recon = [s.to_device(vol)]
    A = s.lfm._fortran_tensor((P, K), "cuda")
    ptrs = (ctypes.c_void_p * 1)(recon[0].data_ptr())
    c = np.asfortranarray(centers)
    ids = np.asfortranarray(neur_id.astype(np.uint8))
    lib_ms = {}
    for fn in ("sid_library", "sid_library_spectral"):
        dst = A if fn == "sid_library" else s.lfm._fortran_tensor((P, K), "cuda")
        times = []
        # the first spectral call also builds the window tap spectra (kept on the plan)
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _lib.call(fn, P_proj._plan, ctypes.cast(ptrs, ctypes.c_void_p), 1, c.ctypes.data,
                      ids.ctypes.data, K, 12, 2.0, dst.data_ptr(), 1, s.lfm._stream_ptr())
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        lib_ms[fn] = {"ms": min(times[1:]), "first_call_ms": times[0]}
        if fn == "sid_library_spectral":
            # FP32 taps against the spectral windows, per library row and overall
            d = torch.linalg.vector_norm(dst - A, dim=0) / torch.linalg.vector_norm(A, dim=0).clamp_min(1e-30)
            lib_ms[fn]["rel_l2_vs_direct"] = float(torch.linalg.vector_norm(dst - A) / torch.linalg.vector_norm(A))
            lib_ms[fn]["rel_l2_vs_direct_worst_row"] = float(d.max())
            del dst
    P_proj.release_workspaces()
    return A, lib_ms


def nnls_inputs(P_proj, K, F):
    """Library generation (library_timing) and the temporal NNLS movie
    Y = S'T + b + noise from it (FP16 and FP32 copies).  Returns (A (P x K,
    L2-normalised columns), Y16, Yf, T_true, library timings)."""
    import torch

    from sid_gb300 import synthetic
    A, lib_ms = library_timing(P_proj, K)
    # L2-normalise library rows (temporal_SID_update.m:42)
    nrm = torch.linalg.vector_norm(A, dim=0)
    A.div_(nrm.clamp_min(1e-30))
    Y16, Yf, T = synthetic.transient_movie(A, F)
    return A, Y16, Yf, T, lib_ms


def nnls_fp64_reference(A, Y16, cols, opts=None):
    """FP64 fast_nnls on the frames `cols` of the FP16 movie: the Gram A'A and
    the cross product A'Y(:, cols) formed in FP64 (torch FP64 products on the
    device, pixel chunks), the iterations by the oracle's FP64 restatement
    (fast_nnls.m:53-199) on the host.  Columns are independent problems, so a
    frame sample checks the whole solve.  Also runs the FP64 solve a second
    time with the normalised Gram formed as diag(h)*Q*diag(h) instead of
    Q./sqrt(diag*diag') (the two differ only in the last bit of some entries):
    the distance between the two FP64 results is the spread that rounding
    alone causes on this problem.  Returns (x64, iterations, x64 of the second
    form, unnormalised FP64 Gram, FP64 cross product)."""
    import numpy as np
    import torch

    from oracle import oracle
    P, K = A.shape
    Q = torch.zeros(K, K, dtype=torch.float64, device=A.device)
    c = torch.zeros(K, len(cols), dtype=torch.float64, device=A.device)
    idx = torch.as_tensor(np.asarray(cols), device=A.device)
    step = 1 << 17
    for p0 in range(0, P, step):
        a = A[p0:p0 + step].double()
        Q += a.T @ a
        c += a.T @ Y16[p0:p0 + step].index_select(1, idx).double()
    Q = Q.cpu().numpy()
    c = c.cpu().numpy()
    dq = np.sqrt(np.diag(Q))
    h = 1.0 / dq
    lam = float((opts or {}).get("lambda", 0.0))
    df = h[:, None] * (-c + lam)
    empty_a, empty_y = np.zeros((0, K)), np.zeros((0, len(cols)))
    xx, _, _, _, it = oracle.fast_nnls(empty_a, empty_y, opts, Q / np.outer(dq, dq), df, h, return_iters=True)
    xx2, _, _, _ = oracle.fast_nnls(empty_a, empty_y, opts, (h[:, None] * Q) * h[None, :], df, h)
    return xx, it, xx2, Q, c


def nnls_accuracy(T, x64, Q, c):
    """Distances of a solve T (K x n frames) from the FP64 solve x64 of the same
    frames: in the iterate (rel-L2), in data space (||A(T - x64)|| / ||A x64||,
    through the FP64 Gram Q = A'A) and in the objective the solve lowers,
    f(t) = t'Qt/2 - c't (= ||y - At||^2/2 up to a constant; max and median
    over frames of |f(T) - f(x64)| / |f(x64)|)."""
    import numpy as np
    D = T - x64
    f = lambda X: 0.5 * np.einsum("kf,kl,lf->f", X, Q, X) - np.einsum("kf,kf->f", c, X)  # noqa: E731
    obj = np.abs(f(T) - f(x64)) / np.abs(f(x64))
    return {"iterate_rel_l2": float(np.linalg.norm(D) / np.linalg.norm(x64)),
            "data_rel_l2": float(np.sqrt(np.einsum("kf,kl,lf->", D, Q, D) / np.einsum("kf,kl,lf->", x64, Q, x64))),
            "objective_rel_max": float(obj.max()), "objective_rel_median": float(np.median(obj))}


def nnls_workload(args, P_proj):
    """Library generation (800 anisotropic Gaussian neurons, sigma_xy U(2,4),
    sigma_z U(1,2), uniform in the 1005^2 x 31 volume) followed by the temporal
    NNLS of 3000 FP16 frames Y = S'T + b + noise (SNR 10), T sparse exponential
    transients (0.5 Hz events at 20 Hz, tau 0.3 s).  Times fast_nnls (the SID
    temporal update, temporal_SID_update.m:45) at split tensor-core precision
    and at FP32, and the Gram / cross contractions on their own; checks both
    solves against FP64 on a frame sample."""
    import numpy as np
    import torch

    import sid_gb300 as s
    K, F = args.nnls_neurons, args.nnls_frames
    P = P_proj.X * P_proj.Y
    A, Y16, Yf, T, lib_ms = nnls_inputs(P_proj, K, F)
    ctx = s.Context()
    out = {"workload": f"library {K} neurons + temporal NNLS {K} x {F} frames, P = {P}, FP16 movie"}
    direct, spec = lib_ms["sid_library"], lib_ms["sid_library_spectral"]
    out["library_ms"] = direct["ms"]
    out["library_neurons_per_s"] = K / (direct["ms"] / 1e3)
    out["library_spectral"] = {
        "ms": spec["ms"], "neurons_per_s": K / (spec["ms"] / 1e3), "first_call_ms": spec["first_call_ms"],
        "speedup_vs_direct": direct["ms"] / spec["ms"], "rel_l2_vs_direct": spec["rel_l2_vs_direct"],
        "rel_l2_vs_direct_worst_row": spec["rel_l2_vs_direct_worst_row"],
        "api": "sid_library_spectral (tensor-core contraction over lenslet-window tap spectra)"}

    def timed(fn, reps=1):
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            r = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps, r

    # contractions alone (with their operand conversions), and the GEMM launches
    # inside them (context timing: CUDA events around the tensor-core kernels)
    ctx.gram(A, "split"); ctx.cross(A, Y16, "split")
    ctx.timing(True)
    ctx.timing_read()
    t_gram, G = timed(lambda: ctx.gram(A, "split"), 3)
    g_ms, g_n = ctx.timing_read()
    t_cross, _ = timed(lambda: ctx.cross(A, Y16, "split"), 3)
    c_ms, c_n = ctx.timing_read()
    ctx.timing(False)
    g_ms /= max(g_n, 1)
    c_ms /= max(c_n, 1)
    t_gram32, G32 = timed(lambda: ctx.gram(A, "fp32"))
    peak = 1929.9
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"])
    except Exception:
        pass
    # the Gram is symmetric: the kernel computes the tiles on and above the diagonal and mirrors
    # them, so the tensor work it needs is 3 passes x K(K+1)P (the triangle), not 3 x 2K^2P
    out["gram_split"] = {"ms": t_gram, "alg_tflops": 2 * K * K * P / t_gram / 1e9,
                         "tensor_tflops_triangle": 3 * K * (K + 1) * P / t_gram / 1e9,
                         "tensor_frac_of_bf16_peak_triangle": 3 * K * (K + 1) * P / t_gram / 1e9 / peak,
                         "rel_l2_vs_fp32": float(torch.linalg.norm(G - G32) / torch.linalg.norm(G32)),
                         "symmetric_max_abs": float((G - G.T).abs().max()),
                         "gemm_ms": g_ms,
                         "gemm_tensor_frac_of_bf16_peak_triangle": 3 * K * (K + 1) * P / g_ms / 1e9 / peak,
                         "note": "ms includes the BF16 hi/lo split of the 800 x 1,010,025 operand (3.2 GB read, "
                                 "3.2 GB written); gemm_ms is the tensor-core launch and its mirror alone"}
    out["cross_split_f16"] = {"ms": t_cross, "alg_tflops": 2 * K * P * F / t_cross / 1e9,
                              "tensor_tflops": 2 * 2 * K * P * F / t_cross / 1e9,
                              "tensor_frac_of_bf16_peak": 2 * 2 * K * P * F / t_cross / 1e9 / peak,
                              "gemm_ms": c_ms,
                              "gemm_tensor_frac_of_bf16_peak": 2 * 2 * K * P * F / c_ms / 1e9 / peak}
    out["gram_fp32_ms"] = t_gram32
    # rank-1 background (bg_iter = 2, sid_main.m:95) + std image (sid_main.m:101) on the
    # FP16 movie: 2 passes over Y per iteration, the std image fused into the last
    hbm = 6707.2
    try:
        hbm = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        pass
    ctx.rank_1_factorization(Y16, 2, std_image=True)
    t_bg, _ = timed(lambda: ctx.rank_1_factorization(Y16, 2, std_image=True), 3)
    bg_bytes = 4 * P * F * 2
    out["background_rank1_std"] = {"ms": t_bg, "passes_over_movie": 4, "bytes": bg_bytes,
                                   "achieved_gbs": bg_bytes / t_bg / 1e6,
                                   "frac_of_hbm": bg_bytes / t_bg / 1e6 / hbm}
    # fast_nnls, split tensor-core precision (FP16 movie) vs the plain FP32 path;
    # one untimed call each first (its CUDA graphs, workspaces and kernel loads
    # cost ~0.25 s once per context), then the mean of the timed calls
    ctx.fast_nnls(A, Y16, {}, prec="split")
    t_split, (Xs, _, its) = timed(lambda: ctx.fast_nnls(A, Y16, {}, prec="split", return_iters=True), 3)
    ctx.fast_nnls(A, Yf, {}, prec="fp32")
    t_fp32, (X32, _, it32) = timed(lambda: ctx.fast_nnls(A, Yf, {}, prec="fp32", return_iters=True), 2)
    out["fast_nnls_split"] = {"ms": t_split, "frames_per_s": F / (t_split / 1e3),
                              "iters_median": float(its.float().median()), "iters_max": int(its.max())}
    out["fast_nnls_fp32"] = {"ms": t_fp32, "frames_per_s": F / (t_fp32 / 1e3),
                             "iters_median": float(it32.float().median()), "iters_max": int(it32.max())}
    out["split_vs_fp32_speedup"] = t_fp32 / t_split
    out["rel_l2_split_vs_fp32"] = float(torch.linalg.norm(Xs - X32) / torch.linalg.norm(X32))
    out["rel_l2_vs_T_true"] = float(torch.linalg.norm(Xs - T) / torch.linalg.norm(T))
    if args.nnls_fp64_frames > 0:
        cols = np.sort(np.random.default_rng(11).choice(F, min(F, args.nnls_fp64_frames), replace=False))
        t0 = time.perf_counter()
        x64, it64, x64b, Q64, c64 = nnls_fp64_reference(A, Y16, cols)
        ci = torch.as_tensor(cols, device=A.device)
        ev = np.linalg.eigvalsh(Q64 / np.sqrt(np.outer(np.diag(Q64), np.diag(Q64))))
        sub = lambda Xg: Xg.index_select(1, ci).double().cpu().numpy()  # noqa: E731
        out["fp64_check"] = {
            "frames": len(cols), "seconds": time.perf_counter() - t0,
            "iters_median": float(np.median(it64)), "iters_max": int(it64.max()),
            "normalised_gram_eig_min_max": [float(ev[0]), float(ev[-1])],
            "split": nnls_accuracy(sub(Xs), x64, Q64, c64),
            "fp32": nnls_accuracy(sub(X32), x64, Q64, c64),
            "fp64_second_rounding": nnls_accuracy(x64b, x64, Q64, c64)}
    # one NMF refinement round on the same factors (fast_NMF.m:185-186): S = the
    # library rows (P x K), T = the temporal NNLS result (K x F), split precision
    ctx.t_update(Y16, Xs, A, {"lamb_temp": 0.01})
    t_tu, _ = timed(lambda: ctx.t_update(Y16, Xs, A, {"lamb_temp": 0.01}), 2)
    ctx.s_update(Y16, A, Xs, {"lamb_spat": 0.01})
    t_su, _ = timed(lambda: ctx.s_update(Y16, A, Xs, {"lamb_spat": 0.01}), 2)
    out["nmf_steps"] = {"T_update_ms": t_tu, "S_update_ms": t_su, "prec": "split",
                        "S_update_tensor_tflop": (2 * P * F * K + 2 * 2 * P * K * K) * 1e-12}
    ctx.sync()
    return out


def demix_workload(args, P_proj):
    """The alternating SID demixing loop (sid_main.m:470-511) on the
    1500-neuron, 5000-frame configuration at 1005^2: neurons and their
    library rows from the projector (generate_LFM_library_GPU.m), square
    support templates of 20-200 lenslets (log-uniform), an FP16 movie
    Y = S'T + b + noise, then per outer iteration the spatial update
    (spatial_SID_update.m:32-33: rows of T normalised, update_spatial_component),
    the temporal update (temporal_SID_update.m:42-47: rows of the forward model
    normalised, fast_nnls warm-started at the previous traces) and merge_filters.
    Times each stage; after the last iteration checks the spatial update at 256
    pixels and the temporal update at 64 frames against FP64 (oracle), and the
    gradient of ||Y - S'T||^2 / 2 from the contractions against central
    differences at 32 entries."""
    import ctypes

    import numpy as np
    import torch

    import sid_gb300 as s
    from oracle import oracle
    from sid_gb300 import _lib, synthetic
    K, F, iters = args.demix_neurons, args.demix_frames, args.demix_iters
    X, Y, Z, N = P_proj.X, P_proj.Y, P_proj.Z, P_proj.Nnum
    P = X * Y
    dev = "cuda"
    vol, centers = synthetic.neuron_volume(X, Y, Z, K, seed=9)
    lib = s.lfm._fortran_tensor((P, K), dev)
    ptrs = (ctypes.c_void_p * 1)(s.to_device(vol).data_ptr())
    c = np.asfortranarray(centers)
    ids = np.ones((K, 1), dtype=np.uint8, order="F")
    _lib.call("sid_library", P_proj._plan, ctypes.cast(ptrs, ctypes.c_void_p), 1, c.ctypes.data, ids.ctypes.data, K, 12,
              2.0, lib.data_ptr(), 1, s.lfm._stream_ptr())
    lib.div_(torch.linalg.vector_norm(lib, dim=0).clamp_min(1e-30))
    # templates: square crops of 20..200 lenslets around each centre
    rng = np.random.default_rng(13)
    area = np.exp(rng.uniform(np.log(20), np.log(200), K))
    half = np.sqrt(area) * N / 2
    tmpl = torch.zeros((P, K), dtype=torch.uint8, device=dev).T  # K x P, column-major (template(k, p))
    tv = tmpl.T.reshape(Y, X, K)  # [y][x][k] view of the same memory
    for k in range(K):
        x0, x1 = max(0, int(centers[k, 0] - half[k])), min(X, int(centers[k, 0] + half[k]) + 1)
        y0, y1 = max(0, int(centers[k, 1] - half[k])), min(Y, int(centers[k, 1] + half[k]) + 1)
        tv[y0:y1, x0:x1, k] = 1
    # movie: S'T (the library restricted to its templates) + background + noise, FP16, pixel chunks
    g = torch.Generator(device=dev).manual_seed(17)
    ev = (torch.rand(K, F, generator=g, device=dev) < 0.025).float() * (0.5 + torch.rand(K, F, generator=g,
                                                                                        device=dev))
    kern = torch.exp(-torch.arange(0, 40, device=dev, dtype=torch.float32) / 6.0)
    T_true = torch.nn.functional.conv1d(ev[:, None, :], kern.flip(0)[None, None, :], padding=39)[:, 0, :F]
    Y16 = torch.empty((F, P), dtype=torch.float16, device=dev).T  # P x F column-major
    S_true = lib * tmpl.T.float()  # P x K, zero outside the templates
    step = 1 << 15
    rms = None
    for p0 in range(0, P, step):
        sig = S_true[p0:p0 + step] @ T_true
        if rms is None:
            rms = float(sig.pow(2).mean().sqrt())
        Y16[p0:p0 + step] = (sig + rms / 10 + rms / 10 * torch.randn(sig.shape, generator=g, device=dev)).half()
    del S_true, sig
    # initial state (sid_main.m before the loop): the library rows and a flat background as the
    # forward model, traces from one temporal NNLS pass without a warm start
    ctx = s.Context()
    fm = torch.cat([lib.T, torch.full((1, P), 1.0 / np.sqrt(P), device=dev)], 0)  # R x P
    Tk, _ = ctx.fast_nnls(s.to_device(fm.T), Y16, {}, prec="split")
    fm = s.to_device(fm)
    kept = K + 1
    del lib

    def ev_t():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def prune(rows_keep, *mats):
        # drop components (the background, last, always stays) and their template rows
        rows_keep = rows_keep.clone()
        rows_keep[-1] = True
        idx = torch.nonzero(rows_keep).flatten()
        return idx, [m.index_select(0, idx[:-1] if m.shape[0] == rows_keep.numel() - 1 else idx) for m in mats]

    stage = {"spatial_ms": [], "temporal_ms": [], "merge_ms": []}
    for it in range(iters):
        e0 = ev_t()
        # spatial_SID_update.m:21-33: drop traces that never exceed 1e-7, normalise, spatial update
        idx, (Tk, tmpl) = prune((Tk > 1e-7).any(dim=1), Tk, tmpl)
        kept = idx.numel()
        Tn = Tk / torch.linalg.vector_norm(Tk, dim=1, keepdim=True).clamp_min(1e-30)
        fm = ctx.spatial_update(Tn, Y16, tmpl, {"bg_sub": 1})
        e1 = ev_t()
        # temporal_SID_update.m:21-47: drop spatial components that never exceed 1e-12, normalise,
        # fast_nnls warm-started at the current traces
        idx, (fm, Tk, tmpl) = prune((fm > 1e-12).any(dim=1), fm, Tk, tmpl)
        kept = idx.numel()
        fmn = fm / torch.linalg.vector_norm(fm, dim=1, keepdim=True).clamp_min(1e-30)
        A = s.to_device(fmn.T)  # P x R, column-major
        Tk, _ = ctx.fast_nnls(A, Y16, {"warm_start": s.to_device(Tk)}, prec="split")
        e2 = ev_t()
        fm, Tk, tm2, _ = s.merge_filters(fmn, Tk, tmpl, np.arange(kept), {"limit": 0.9, "bg_sub": 1})
        tmpl = tm2.to(torch.uint8)
        kept = Tk.shape[0]
        e3 = ev_t()
        torch.cuda.synchronize()
        stage["spatial_ms"].append(e0.elapsed_time(e1))
        stage["temporal_ms"].append(e1.elapsed_time(e2))
        stage["merge_ms"].append(e2.elapsed_time(e3))
        del A
    out = {"workload": f"demixing loop {K} neurons x {F} frames at {X}x{Y} (FP16 movie), {iters} outer iterations, "
                       f"templates of 20-200 lenslets",
           "components_after": int(kept),
           "seconds_per_outer_iteration": float(np.mean([a + b + c_ for a, b, c_ in zip(
               stage["spatial_ms"], stage["temporal_ms"], stage["merge_ms"])]) / 1e3)}
    out.update({k: [round(v, 2) for v in vals] for k, vals in stage.items()})
    # FP64 checks after the last iteration
    idx, (Tk, tmpl) = prune((Tk > 1e-7).any(dim=1), Tk, tmpl)
    kept = idx.numel()
    Tn = Tk / torch.linalg.vector_norm(Tk, dim=1, keepdim=True).clamp_min(1e-30)
    fm_last = ctx.spatial_update(Tn, Y16, tmpl, {"bg_sub": 1})
    torch.cuda.synchronize()
    tm_np = tmpl
    cover = torch.nonzero(tm_np.sum(dim=0) > 0).flatten().cpu().numpy()
    pix = np.sort(rng.choice(cover, 256, replace=False))
    Tn64 = Tn.double().cpu().numpy()
    errs_num, errs_den = 0.0, 0.0
    ncomp = []
    for p in pix:
        idx = np.append(np.flatnonzero(tm_np[:, int(p)].cpu().numpy()), kept - 1)
        ncomp.append(len(idx))
        yv = Y16[int(p)].double().cpu().numpy()
        nrm = np.linalg.norm(yv)
        ref = oracle.reg_nnls(Tn64[idx].T, yv / nrm, {"bg_sub": 1}) * nrm
        got = fm_last[torch.as_tensor(idx, device=dev), int(p)].double().cpu().numpy()
        errs_num += float(np.sum((got - ref) ** 2))
        errs_den += float(np.sum(ref ** 2))
    out["spatial_vs_fp64_256px"] = {"rel_l2": float(np.sqrt(errs_num / max(errs_den, 1e-300))),
                                     "components_per_pixel_max": int(max(ncomp)),
                                     "components_per_pixel_median": float(np.median(ncomp))}
    # temporal update at 64 frames: the same warm-started solve in FP64
    idx, (fm_last, Tk) = prune((fm_last > 1e-12).any(dim=1), fm_last, Tk)
    kept = idx.numel()
    fmn = fm_last / torch.linalg.vector_norm(fm_last, dim=1, keepdim=True).clamp_min(1e-30)
    A = s.to_device(fmn.T)
    W = Tk.clone()
    Tg, _ = ctx.fast_nnls(A, Y16, {"warm_start": s.to_device(W)}, prec="split")
    cols = np.sort(rng.choice(F, 64, replace=False))
    ci = torch.as_tensor(cols, device=dev)
    Q = torch.zeros(kept, kept, dtype=torch.float64, device=dev)
    cr = torch.zeros(kept, len(cols), dtype=torch.float64, device=dev)
    for p0 in range(0, P, 1 << 16):
        a = A[p0:p0 + (1 << 16)].double()
        Q += a.T @ a
        cr += a.T @ Y16[p0:p0 + (1 << 16)].index_select(1, ci).double()
    Q, cr = Q.cpu().numpy(), cr.cpu().numpy()
    dq = np.sqrt(np.diag(Q))
    h = 1.0 / dq
    Wc = W.index_select(1, ci).double().cpu().numpy()
    x64, *_ = oracle.fast_nnls(np.zeros((0, kept)), np.zeros((0, len(cols))), {"warm_start": Wc},
                               Q / np.outer(dq, dq), h[:, None] * (-cr), h)
    out["temporal_vs_fp64_64frames"] = nnls_accuracy(Tg.index_select(1, ci).double().cpu().numpy(), x64, Q, cr)
    # gradient of ||Y - A T||^2 / 2 wrt T from the contractions vs central differences (FP64), away
    # from the minimiser (at the NNLS solution the passive entries' gradient is rounding noise)
    G = ctx.gram(A, "split").double()
    C = ctx.cross(A, Y16, "split").double()
    Tg = 1.5 * Tg + 0.05 * Tg.mean()
    grad = G @ Tg.double() - C
    ent = np.stack([rng.integers(0, kept, 32), rng.integers(0, F, 32)], 1)
    fd, gv = [], []
    for k, f in ent:
        yv = Y16[:, int(f)].double()
        t = Tg[:, int(f)].double()
        r = yv.clone()
        for p0 in range(0, P, 1 << 17):
            r[p0:p0 + (1 << 17)] -= A[p0:p0 + (1 << 17)].double() @ t
        a = A[:, int(k)].double()
        hh = 1e-3 * max(abs(float(t[int(k)])), 1e-3)
        fp = 0.5 * torch.sum((r - hh * a) ** 2)
        fm_ = 0.5 * torch.sum((r + hh * a) ** 2)
        fd.append(float((fp - fm_) / (2 * hh)))
        gv.append(float(grad[int(k), int(f)]))
    fd, gv = np.array(fd), np.array(gv)
    out["gradient_vs_central_differences_32"] = float(np.linalg.norm(gv - fd) / np.linalg.norm(fd))
    return out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    H, V = workload(args.config)
    nthreads = os.cpu_count() or 1
    per = []
    cols = 0
    measured = 0.0
    budget = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    for i in range(args.warmup + args.steps):
        t_proj, cols, spent = cpu_sample(H, V, budget, nthreads)
        if i >= args.warmup:
            per.append(2.0 * t_proj)  # one RL iteration = forward + back projection
            measured += spent
    t_iter = statistics.median(per)
    value = 1.0 / t_iter
    sample = (f"FP32 lenslet-sparse forward projection (oracle/sid_oracle.c baseline_forward_f32) on {cols} of "
              f"{V.shape[1]} sensor columns per step, extrapolated linearly to all columns; one RL iteration "
              f"= 2 projections (forward + equal-cost back projection)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_iter * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(V.shape[0], V.shape[1], V.shape[2], H.shape[2],
                                                 H.shape[0]),
                       "parallelism": "host cores (OpenMP)"},
            "extrapolated": True,
            "sampled_sensor_columns_per_step": cols,
            "measured_cpu_seconds": measured,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch

    import sid_gb300 as s
    from oracle import oracle

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    H, Vt = workload(args.config, args.depths)
    X, Y, Z = Vt.shape
    methods = [args.method] + [m for m in args.compare.split(",") if m and m != args.method]
    plan_methods = list(methods)
    if not args.no_nnls and "direct" not in plan_methods:
        plan_methods.append("direct")  # the library generation reads the lenslet taps
    # the tensor-core batched projections need the transposed 24-bit spectra
    tc = args.method == "spectral_mixed" and args.batch_volumes > 1 and not args.library_only
    if args.library_only:
        plan_methods = ["direct"]  # both library forms read only the lenslet taps
    P = s.Projector(H, (X, Y), None, methods=tuple(plan_methods), batched=tc)
    info = P.info()
    if args.library_only:
        _, lib = library_timing(P, args.nnls_neurons)
        if rank == 0:
            print(json.dumps({"workload": f"library {args.nnls_neurons} neurons (neur_rad 12, axial 2) at "
                                          f"{X}x{Y}x{Z}", "library": lib}))
        return 0
    # RL input: Htf = A^T y with y = A V_true (the reference starts ISRA at Xguess = Htf)
    y = P.forward(Vt, method=args.method)
    Htf = P.adjoint(y, method=args.method)
    X0 = Htf.clone()
    torch.cuda.synchronize()

    def iterate(x, m, k):
        # k ISRA iterations in one deconvRL call (the reference runs maxIter = 8..30
        # iterations per call, reconstruct_S.m:195): the volume <-> polyphase
        # conversions happen once per call, every iteration is a full step
        from sid_gb300 import _lib
        _lib.call("sid_deconv_isra", P._plan, _lib.METHODS[m], Htf.data_ptr(), x.data_ptr(), k, 0.0,
                  s.lfm._stream_ptr())

    x = X0.clone()
    iterate(x, args.method, args.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    P.timing(True)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        iterate(x, args.method, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    P.timing(False)
    ms = e0.elapsed_time(e1)
    k_ms, k_n = P.timing_read()
    P.sync()
    ms, value = replica_throughput(ms, args.steps, world, "cuda")
    ms_per_step = ms / args.steps

    # roofline of the dominant kernel (the spectral contraction streams the tap spectra)
    n_out, n_in = info["Nnum"] ** 2, info["Nnum"] ** 2 * info["Z"]
    nf = (info["L"] // 2 + 1) * info["L"]
    hbm, peak_kind = peaks()
    roof = None
    esz = {"spectral_f32": (8, 8), "spectral_i16": (4, 4), "spectral_mixed": (4, 6), "spectral_mixed_f32": (4, 8)}
    ws_gb = nf * n_out * n_in * sum(esz.get(args.method, (0, 0))) / 1e9
    if args.method == "direct":
        ws_gb = info["device_bytes"] / 1e9  # the lenslet taps and workspaces
    if args.method.startswith("spectral") and k_n:
        # per step one forward and one back-projection contraction; each streams its
        # tap spectra once (bytes per complex entry: 16-bit block float 4, 24-bit float 6, FP32 8)
        esz_f, esz_b = esz[args.method]
        alg_bytes = (nf * n_out * n_in * (esz_f + esz_b) + 2 * nf * (n_in + n_out) * 8) / 2
        avg_s = k_ms / k_n / 1e3
        achieved = alg_bytes / avg_s / 1e9
        traffic = None
        tf = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tf):
            rec = json.load(open(tf))
            if rec.get("volume") == [X, Y, Z]:  # captured on this volume size only
                traffic = rec.get(f"k_spec_{args.method}")
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "kernel": "k_spec_fwd/k_spec_adj (tap-spectra contraction)",
                "launches": k_n, "avg_launch_ms": k_ms / k_n, "algorithmic_bytes_per_launch": alg_bytes,
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)"}

    # end to end: the host-array ISRA entry point (copies inside the timed region)
    def pinned_copy(t):
        a = s.to_numpy(t)
        buf = torch.empty(a.size, dtype=torch.float32, pin_memory=True).numpy()
        out = buf.reshape(a.shape, order="F")
        out[...] = a
        return out

    xh = pinned_copy(X0)
    hh = pinned_copy(Htf)
    P.isra_host(hh, xh, 1, method=args.method)
    t0 = time.perf_counter()
    e2e_steps = max(3, args.steps // 4)
    for _ in range(e2e_steps):
        P.isra_host_inplace(hh, xh, 1, method=args.method)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    vol_bytes = X * Y * Z * 4

    # accuracy of the timed method: forward projection vs the FP64 oracle at 256 sampled pixels
    rng = np.random.default_rng(0)
    pix = np.stack([rng.integers(0, X, 256), rng.integers(0, Y, 256)], 1)
    ref_pix = oracle.forward_project_pixels(H, Vt, pix)
    got = s.to_numpy(P.forward(Vt, method=args.method))[pix[:, 0], pix[:, 1]]
    fwd_err = float(np.linalg.norm(got - ref_pix) / np.linalg.norm(ref_pix))

    # other methods (fewer steps, same workload) for the mixed-vs-FP32 comparison
    others = {}
    for m in methods[1:]:
        xm = X0.clone()
        iterate(xm, m, 1)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        iterate(xm, m, args.compare_steps)
        b.record(stream)
        torch.cuda.synchronize()
        tm = a.elapsed_time(b) / args.compare_steps
        gm = s.to_numpy(P.forward(Vt, method=m))[pix[:, 0], pix[:, 1]]
        others[m] = {"rl_iter_s": 1e3 / tm, "ms_per_iter": tm,
                     "fwd_rel_err_vs_fp64": float(np.linalg.norm(gm - ref_pix) / np.linalg.norm(ref_pix))}

    # neuron-kernel composition (reconstruct_S.m:126-127): ISRA iterations with
    # convn(., k, 'same') before every forward and after every back projection
    composed = {}
    for kname, ker in (("ball_3_1", s.generate_kernel("ball", [3, 1])),
                       ("gaussian_17x17x5", s.generate_kernel("gaussian", [1.6, 0.8]))):
        P.set_kernel(ker)
        xk = X0.clone()
        iterate(xk, args.method, 2)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        iterate(xk, args.method, 5)
        b.record(stream)
        torch.cuda.synchronize()
        tk = a.elapsed_time(b) / 5
        composed[kname] = {"kernel": list(ker.shape), "rl_iter_s": 1e3 / tk, "ms_per_iter": tk,
                           "overhead_ms_per_iter": tk - ms_per_step}
        P.set_kernel(None)
        del xk

    # several components per pass over the tap spectra (reconstruct_S.m:162-212): nbv volumes, 3 ISRA
    # iterations each, against the same iterations one volume at a time.  With the tensor-core plan the
    # mixed form contracts up to 64 volumes per pass (spec_tc.cu, as many as the free device memory holds
    # workspaces for); other methods 4 per pass on the FP32 pipes.
    batched = None
    if args.method.startswith("spectral") and args.batch_volumes > 1:
        nbv = args.batch_volumes
        hs = [Htf.clone() for _ in range(nbv)]
        xs = [X0.clone() for _ in range(nbv)]
        P.isra_batched(hs, xs, 1, method=args.method)  # sizes the workspaces
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        P.timing(True)
        a.record(stream)
        outs = P.isra_batched(hs, xs, 3, method=args.method)
        b.record(stream)
        torch.cuda.synchronize()
        P.timing(False)
        tb = a.elapsed_time(b)
        kb_ms, kb_n = P.timing_read()
        single = s.to_numpy(P.isra(Htf, X0, 3, method=args.method))
        dev_b = float(np.linalg.norm(s.to_numpy(outs[-1]) - single) / np.linalg.norm(single))
        nf_ = (info["L"] // 2 + 1) * info["L"]
        n_in_, n_out_ = info["Nnum"] ** 2 * info["Z"], info["Nnum"] ** 2
        per_vi = tb / (nbv * 3)
        batched = {"volumes": nbv, "iterations": 3, "ms": tb,
                   "volume_iterations_per_s": 1e3 / per_vi,
                   "components_per_s": 1e3 / per_vi / 8,
                   "components_per_s_note": "components deconvolved per second at reconstruct_S's 8 ISRA "
                                            "iterations per component (reconstruct_S.m:87-89)",
                   "ms_per_volume_iteration": per_vi,
                   "single_volume_ms_per_iteration": ms_per_step,
                   "speedup_per_volume": ms_per_step / per_vi,
                   "rel_l2_last_volume_vs_single_calls": dev_b}
        avg = kb_ms / max(kb_n, 1)
        if tc:
            # tensor-core contraction: launches alternate forward (rows 225, reduction 2 x 6976) and
            # back projection (rows 6976, reduction 2 x 232); 5 BF16 passes per MMA tile
            # volumes per pass, from the launch count (two contractions per iteration and group)
            groups = max(1, kb_n // 6)
            g = -(-nbv // groups)
            bn = 64 if g <= 32 else 128
            nip = -(-n_in_ // 8) * 8
            op = -(-n_out_ // 8) * 8
            kf, ka = 2 * nip, 2 * op
            cd = lambda a_, b_: -(-a_ // b_) * b_  # noqa: E731
            mma_f = 2 * 5 * cd(n_out_, 128) * bn * cd(kf, 64) * nf_
            mma_a = 2 * 5 * cd(nip, 128) * bn * cd(ka, 64) * nf_
            bytes_f = nf_ * n_out_ * kf * 3 + nf_ * bn * kf * 6 + nf_ * g * n_out_ * 8
            bytes_a = nf_ * nip * ka * 3 + nf_ * bn * ka * 6 + nf_ * g * nip * 8
            bf16_peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]) \
                if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
            batched["contraction"] = {
                "kernel": "k_spec_tc (tcgen05, 24-bit spectra as exact BF16 hi+lo, B split BF16 hi/mid/lo, "
                          "5 passes)",
                "volumes_per_pass": g, "launches": kb_n, "avg_launch_ms": avg,
                "tensor_tflops": (mma_f + mma_a) / 2 / (avg / 1e3) / 1e12,
                "tensor_frac_of_bf16_peak": (mma_f + mma_a) / 2 / (avg / 1e3) / 1e12 / bf16_peak,
                "algorithmic_bytes_per_launch": (bytes_f + bytes_a) / 2,
                "hbm_gbs": (bytes_f + bytes_a) / 2 / (avg / 1e3) / 1e9,
                "hbm_frac": (bytes_f + bytes_a) / 2 / (avg / 1e3) / 1e9 / hbm,
                "limit": "shared-memory operand reads of the MMAs (neither DRAM nor the tensor pipe saturated)",
                "peaks": "measured bf16_tflops / hbm_gbs (MEASURED_PEAKS.json)"}
        else:
            flop_launch = 8.0 * nf_ * n_in_ * n_out_ * min(4, nbv)
            fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
            batched["contraction"] = {"kernel": "k_spec_fwd_b/k_spec_adj_b (FP32 pipes, 4 volumes per pass)",
                                      "launches": kb_n, "avg_launch_ms": avg,
                                      "fp32_tflops": flop_launch / avg / 1e9,
                                      "frac_of_fp32_fma_peak": flop_launch / avg / 1e9 / fp32_peak,
                                      "fp32_peak_note": "152 SMs x 128 lanes x 2 FLOP x 2.07 GHz (nominal)"}
        del hs, xs, outs
        P.release_workspaces()
        torch.cuda.empty_cache()

    nnls = None
    if not args.no_nnls:
        nnls = nnls_workload(args, P)
        torch.cuda.empty_cache()
    demix = None
    if not args.no_demix and not args.no_nnls:
        demix = demix_workload(args, P)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        t_proj, cols, _ = cpu_sample(H, Vt, args.cpu_seconds, os.cpu_count() or 1)
        cpu = {"value": 1.0 / (2.0 * t_proj), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"FP32 lenslet-sparse forward projection (oracle/sid_oracle.c) on {cols}/{Y} sensor "
                         f"columns, extrapolated; RL iteration = 2 projections"}

    if rank == 0:
        # per iteration: direct 4 (two projections with their depth reductions) or spectral 6
        # (r2c, contraction, c2r for each projection), plus the ISRA update; 3 layout kernels per call
        # spectral: r2c, forward contraction, c2r, r2c, back-projection contraction,
        # c2r, update, plus the exact recomputation of the weakly observed voxels
        launches_per_iter = 4 if args.method == "direct" else 7 + info.get("weak_launches", 0)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"spectral_i16": "f32 (16-bit block-float spectra)",
                                           "spectral_mixed": "f32 (16-bit forward / 24-bit float back-projection spectra)",
                                           "spectral_mixed_f32": "f32 (16-bit forward / FP32 back-projection spectra)"}
            .get(args.method, "f32"),
            "data": "synthetic (seeded Gaussian PSF + blob volume, shapes of the 1005^2x31 configuration)",
            "config": {"workload": workload_name(X, Y, Z, info["Nnum"], info["M"]),
                       "method": args.method, "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "per-iteration working set (tap spectra streamed once per projection, "
                             f"{ws_gb:.1f} GB per iteration) "
                             "exceeds L2; no flush needed"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * vol_bytes,
                    "d2h_bytes_per_step": vol_bytes,
                    "api": "sid_deconv_isra_host (pinned host arrays, maxIter=1 per step)"},
            "gpu_launches": launches_per_iter * args.steps + 3,
            "clocks": clk.summary(),
            "accuracy": {"fwd_rel_l2_vs_fp64_256px": fwd_err},
            "compare": others,
            "kernel_composition": composed,
            "mixed_vs_fp32_direct": (value / world) / others["direct"]["rl_iter_s"] if "direct" in others else None,
            # the same spectral algorithm with FP32 tap spectra: the speed-up precision alone buys
            "mixed_vs_fp32_spectral": ((value / world) / others["spectral_f32"]["rl_iter_s"]
                                       if "spectral_f32" in others else None),
            "plan": {"L": info["L"], "D": info["D"], "device_gb": info["device_bytes"] / 1e9},
            "batched_components": batched,
            # the mixed-precision batched form per volume-iteration against the FP32 paths one volume at a time
            "batched_mixed_vs_fp32": ({m: (1e3 / batched["ms_per_volume_iteration"]) / others[m]["rl_iter_s"]
                                       for m in ("spectral_f32", "direct") if m in others}
                                      if batched else None),
            "nnls": nnls,
            "demix": demix,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
