#!/usr/bin/env python3
"""Benchmark of the RVGP pipeline on one GB300: fit + predict wall time.

Workload (default): torus R=1, r=0.35, n=20000 points with N(0, 0.01²) jitter,
k=20, m=200 eigenpairs; field = rotational ∂/∂φ + a smoothed random field
(t=50); train on a seeded 30 % (the fit's own 80/20 split inside, as in the
reference), 200 Adam steps on the log marginal likelihood with the
hand-written adjoint, predict mean and variance at the remaining 70 %.

A step = the whole pipeline from points to posterior: kNN graph, gauges,
connections, Laplacians, eigenpairs of L and Lc, lift, GP fit, GP predict.
``value`` = seconds per step of the mixed-precision form with inputs resident
in HBM (CUDA events on the launching stream, L2 flushed between steps).
``fp64_form_s`` = the same step in the plain FP64 form; ``pred_rel_err`` = the
relative L2 difference of the two forms' posterior means.  ``e2e`` = the same
step through the public API with host numpy inputs and outputs.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --model sgpr [--inducing M] [--sgpr-iters I]   # the sparse inducing-point GP
    python bench.py --model rbf [--sgpr-iters I]                    # kernel='rbf' GP
    python bench.py --model features                                # div/curl vector-field features
    python bench.py --model fields                                  # many fields at shared training points
"""
import os

_THREADS = str(os.cpu_count() or 1)
for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, _THREADS)

import argparse  # noqa: E402
import json  # noqa: E402
import subprocess  # noqa: E402
import sys  # noqa: E402
import threading  # noqa: E402
import time  # noqa: E402

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the metric's configuration: Swiss roll in R^64, n = 100000, k = 15, m = 500,
    # 20 % train; d = 2 as configured (the explained-variance estimate is not
    # used: 64-dimensional noise of 0.02 spreads the local variance)
    "swissroll64_n100000_k15_m500": dict(kind="swissroll64", n=100000, D=64, k=15, m=500, train_frac=0.2,
                                         t_smooth=50.0, adam=200, rotational=False, dim=2),
    "torus_n20000_k20_m200": dict(kind="torus", n=20000, D=3, k=20, m=200, train_frac=0.3, t_smooth=50.0, adam=200,
                                  rotational=True),
    # scale-up: a bumpy sphere of 500 000 points, furthest-point sampled on
    # the GPU to 250 000 inside the step, then k = 20, m = 1000, 20 % train
    "bumpy_sphere_n500000_fps250000_k20_m1000": dict(kind="bumpy_sphere", n=250000, n_raw=500000, D=3, k=20,
                                                     m=1000, train_frac=0.2, t_smooth=50.0, adam=200,
                                                     rotational=False, dim=2),
    # the Swiss roll at half size (profiling captures of the wide kernels)
    "swissroll64_n50000_k15_m500": dict(kind="swissroll64", n=50000, D=64, k=15, m=500, train_frac=0.2,
                                        t_smooth=50.0, adam=200, rotational=False, dim=2),
    "sphere_n2000_k10_m50": dict(kind="sphere", n=2000, D=3, k=10, m=50, train_frac=0.5, t_smooth=100.0, adam=200,
                                 rotational=False),
}
DEFAULT_WORKLOAD = "swissroll64_n100000_k15_m500"
METRIC = "RVGP fit+predict wall s (mixed vs FP64 GPU, equal pred. error); HBM GB/s"


def make_inputs(wl, seed=0):
    """Points (the raw cloud when the step samples it first), train / test
    indices into the points the pipeline runs on."""
    from rvgp_gb300.workloads import make_points, rotational_field, split
    X = make_points(wl["kind"], wl.get("n_raw", wl["n"]), seed=seed)
    train, test = split(wl["n"], wl["train_frac"], seed=seed)
    return X, train, test


def sample_points(X, wl):
    """The step's furthest-point sample (RVGP/geometry.py:126-162) when the
    workload starts from a larger cloud: the first wl['n'] points of the FPS
    order from point 0, on the device."""
    if "n_raw" not in wl:
        return X
    import torch
    from rvgp_gb300 import _core
    Xd = X if isinstance(X, torch.Tensor) else torch.as_tensor(X, device="cuda")
    perm, _ = _core.fps(Xd, N=wl["n"], start_idx=0)
    return Xd[perm.long()].contiguous()


def dim_kwargs(wl):
    """Manifold dimension as configured (d = 2) where the workload fixes it."""
    return dict(dim_man=wl["dim"], estimate_dim=False) if "dim" in wl else {}


def bench_config(wl, args, world):
    """The `config` of both arms' JSON lines (identical by construction)."""
    return {"workload": args.workload, "n": wl["n"], "D": wl["D"], "k": wl["k"], "m": wl["m"],
            "train_frac": wl["train_frac"], "adam_steps": wl["adam"], "parallelism": f"replicas{world}",
            "l2": "flushed between steps (256 MiB write)"}


def make_field(X, wl, seed=0):
    """Ground-truth field (outside the timed region): smoothed random tangent
    field (+ the rotational field on the torus)."""
    import rvgp_gb300 as RVGP
    from rvgp_gb300.workloads import rotational_field
    X = sample_points(X, wl)
    d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False, **dim_kwargs(wl))
    d.random_vector_field(seed=seed)
    d.smooth_vector_field(t=wl["t_smooth"])
    v = d.vectors
    if wl["rotational"]:
        import torch
        from rvgp_gb300 import _core
        rot = torch.as_tensor(rotational_field(X), device="cuda")
        rot = _core.frame_map(d._dev.T, d.dim_man, rot, "project")
        v = v + rot.cpu().numpy()
    d.wait()
    return np.ascontiguousarray(v)


# ------------------------------------------------------------------------------ our arm
def pipeline(X, V, train, test, wl, precision, timings=None, keep=None, nvtx=None):
    """One step through the public API; returns (mean, var) on the device
    (with ``keep`` a dict, also the data object and the fitted model)."""
    import torch
    import rvgp_gb300 as RVGP
    if "n_raw" in wl:
        e_fps = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e_fps[0].record()
        X = sample_points(X, wl)
        e_fps[1].record()
        if timings is not None:
            torch.cuda.synchronize()
            timings["fps"] = e_fps[0].elapsed_time(e_fps[1]) / 1e3
    d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], precision=precision, verbose=False,
                                timings=timings, nvtx=nvtx, **dim_kwargs(wl))
    d.vectors = V
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    gp = RVGP.fit(d, train_ind=train, epochs=wl["adam"], optimizer="adam", lr=0.05, verbose=False)
    ev[1].record()
    out = gp.predict_points(test)
    d.wait()  # the concurrent eigensolve of L belongs to the step
    ev[2].record()
    if timings is not None:
        torch.cuda.synchronize()
        timings["gp_fit"] = ev[0].elapsed_time(ev[1]) / 1e3
        timings["gp_predict"] = ev[1].elapsed_time(ev[2]) / 1e3
        timings["eig_L_info"] = d._dev.eig_info_L
        timings["eig_Lc_info"] = d._dev.eig_info_Lc
        timings["gp_fit_form"] = getattr(gp, "fit_form", None)
    if keep is not None:
        keep.update(data=d, model=gp)
    return out


def error_statements(mixed, fp64, mean_mixed, mean64):
    """The mixed form's results against the FP64 form's on the same inputs:
    eigenvalue relative error (Lc and L; over the eigenvalues above 1e-6 of the
    largest, as the null eigenvalue of L is 0, with the largest absolute
    error over the largest eigenvalue beside it), the largest principal-angle sine
    between eigen-subspaces per cluster of numerically equal eigenvalues (the
    eigenvectors inside a cluster are arbitrary) and over the whole m-space,
    the relative L2 error of the posterior mean, and |ΔLML| at each form's
    fitted parameters (FP64 evaluations)."""
    import torch
    da, db = mixed["data"]._dev, fp64["data"]._dev
    mixed["data"].wait()
    fp64["data"].wait()

    def sines(Ua, Ub, ev):
        Qa = Ua / torch.linalg.vector_norm(Ua, dim=0)
        Qb = Ub / torch.linalg.vector_norm(Ub, dim=0)
        ev = ev.cpu().numpy()
        worst, start = 0.0, 0
        for i in range(1, len(ev) + 1):
            if i == len(ev) or abs(ev[i] - ev[i - 1]) > 1e-6 * max(1.0, abs(ev[i])):
                if i < len(ev):  # a cluster cut by the m-th eigenvalue is not comparable
                    s = torch.linalg.svdvals(Qa[:, start:i].T @ Qb[:, start:i])
                    worst = max(worst, float(torch.sqrt(torch.clamp(1 - s.min() ** 2, min=0))))
                start = i
        s_all = torch.linalg.svdvals(Qa.T @ Qb)
        return worst, float(torch.sqrt(torch.clamp(1 - s_all.min() ** 2, min=0)))

    out = {}
    for tag, ea, eb, Ua, Ub in (("Lc", da.evals_Lc, db.evals_Lc, da.evecs_Lc_local, db.evecs_Lc_local),
                                ("L", da.evals_L, db.evals_L, da.evecs_L, db.evecs_L)):
        # relative error over the eigenvalues above 1e-6 of the largest (the
        # null eigenvalue of L is 0 up to rounding), and the largest absolute
        # error in units of the largest returned eigenvalue
        big = eb.abs() >= 1e-6 * float(eb.abs().max())
        rel = float(((ea - eb).abs()[big] / eb.abs()[big]).max())
        absn = float((ea - eb).abs().max() / eb.abs().max())
        cl, whole = sines(Ua, Ub, eb)
        out[f"eigenvalue_rel_err_{tag}"] = rel
        out[f"eigenvalue_abs_err_over_max_{tag}"] = absn
        out[f"principal_angle_sin_max_per_cluster_{tag}"] = cl
        out[f"principal_angle_sin_whole_space_{tag}"] = whole
    out["posterior_mean_rel_err"] = float(torch.linalg.vector_norm(mean_mixed - mean64) /
                                          torch.linalg.vector_norm(mean64))
    la, lb = mixed["model"].log_marginal_likelihood(), fp64["model"].log_marginal_likelihood()
    out["abs_delta_lml"] = abs(la - lb)
    out["rel_delta_lml"] = abs(la - lb) / abs(lb)
    out["theta_mixed"] = [float(v) for v in mixed["model"].theta().cpu().numpy()]
    out["theta_fp64"] = [float(v) for v in fp64["model"].theta().cpu().numpy()]
    return out


def flush_l2(buf):
    buf.add_(1.0)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.active", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# chunked Chebyshev-step SpMM, keyed by (n, d, p, stored blocks) of the
# workload's Lc, with where the figure comes from.  The capture was made on
# the n = 50 000 Swiss roll (profiles/bspmm_chunked_kernel_f32_Lc_
# swissroll64_n50000_p564.md: 693.6 MB against 694.8 MB algorithmic); every
# term of the product's traffic (X and Z read, Y written, blocks and column
# indices) grows with the rows and stored blocks, so at n = 100 000 it is
# scaled by the algorithmic bytes, 1 389 591 924 / 694 757 164.
SPMM_TRAFFIC = {
    (100000, 2, 564, 1779596): (int(693.6e6 * 1389591924 / 694757164),
                                "ncu capture at n = 50 000, scaled by the units processed"),
    (50000, 2, 564, 887858): (int(693.6e6), "ncu capture"),
}


def spmm_roofline(d, wl, peaks, flush, reps=20):
    """Achieved HBM bandwidth of the eigensolver's Chebyshev-step SpMM (FP32,
    block width p) on this workload's connection Laplacian: each launch timed
    alone with CUDA events on the launching stream, L2 flushed before it.  The
    matrix is the Morton-renumbered one the eigensolver multiplies by, and the
    product the launch tuner's variant (what the eigensolver runs); the
    product through the matrix's plan (the tuner then also tries the grouped
    and tiled forms) is timed beside it for reference."""
    import torch
    from rvgp_gb300 import _core
    dev = d._dev
    ip, ix, _, v32 = _core.permute_csr(dev.indptr, dev.indices, dev.Lc_vals, dev.Lc_vals32, dev.perm, dev.rank)
    n, k = d.n, d.dim_man
    N = n * k
    p = _core.block_size(wl["m"], N)
    plan = _core.spmm_plan(ip, ix, k)
    torch.cuda.nvtx.range_push("spmm_roofline")  # lets a profiler select exactly these launches
    X = torch.randn((N, p), dtype=torch.float32, device="cuda")
    Z = torch.randn_like(X)
    Y = torch.empty_like(X)
    s = torch.cuda.current_stream()

    def timed(pl):
        for _ in range(50):  # untimed: clocks up, tuner choice made
            _core.bspmm(ip, ix, v32, X, Y, Z, 0.1, -0.2, 0.3, plan=pl)
        times = []
        for _ in range(reps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            _core.bspmm(ip, ix, v32, X, Y, Z, 0.1, -0.2, 0.3, plan=pl)
            e1.record(s)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        return float(np.mean(times))

    t = timed(None)  # the variant the launch tuner picked for this shape (what the eigensolver runs)
    torch.cuda.nvtx.range_pop()
    t_plan = timed(plan)
    key = f"bspmm f32 DB{k} b{p} n2^{int(n).bit_length() - 1}".encode()
    variant = int(_core.lib().rvgp_autotune_lookup(key))
    E = dev.indices.numel()
    # values + column indices + row pointers + read X, read Z, write Y
    alg = E * (k * k * 4 + 4) + (n + 1) * 4 + 3 * N * p * 4
    achieved = alg / t / 1e9
    names = {0: f"bspmm_kernel<float,{k},G>", 1: f"bspmm_chunked_kernel<float,{k},2>",
             2: f"bspmm_chunked_kernel<float,{k},4>", 3: f"bspmm_tile_kernel<float,{k},2>",
             4: f"bspmm_tile_kernel<float,{k},4>", 5: f"bspmm_chunked_kernel<float,{k},2,L2>",
             6: f"bspmm_tile_kernel<float,{k},2,L2>", 7: f"bspmm_chunked_kernel<float,{k},2,rowblocks>",
             8: f"bspmm_tiled_kernel<float,{k},2>", 9: f"bspmm_group_kernel<float,{k},2>",
             10: f"bspmm_group_kernel<float,{k},1>"}
    return {"kernel": f"{names.get(variant, '?')} (Chebyshev step, Lc x block; launch tuner's variant {variant})",
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4),
            "traffic": SPMM_TRAFFIC.get((n, k, p, E), (None, None))[0],
            "traffic_source": SPMM_TRAFFIC.get((n, k, p, E), (None, None))[1], "algorithmic_bytes": int(alg),
            "avg_launch_us": round(t * 1e6, 2), "planned_avg_launch_us": round(t_plan * 1e6, 2),
            "block_width": p, "l2": "flushed before every timed launch"}


def run_ours(args):
    import torch
    import torch.distributed as dist
    from rvgp_gb300 import _core

    from rvgp_gb300 import replicas

    rank, world, local = replicas.world()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    _core.require_cuda()
    wl = WORKLOADS[args.workload]
    seed = replicas.replica_seed(0, rank)  # rank 0 uses seed 0, the reference arm's inputs
    X, train, test = make_inputs(wl, seed=seed)
    V = make_field(X, wl, seed=seed)
    Xd = torch.as_tensor(X, device="cuda")
    Vd = torch.as_tensor(V, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        pipeline(Xd, Vd, train, test, wl, "mixed")
    barrier()
    stream = torch.cuda.current_stream()
    times = []
    launches0 = _core.launch_count()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.nvtx.range_push("timed_step")  # lets a profiler select exactly these launches
            e0.record(stream)
            mean_mixed, _ = pipeline(Xd, Vd, train, test, wl, "mixed", nvtx="timed_step")
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            barrier()
            times.append(e0.elapsed_time(e1) / 1e3)
    launches = _core.launch_count() - launches0
    t_step = float(np.mean(times))
    stages = {}
    kept_mixed = {}
    # untimed step with a per-stage breakdown (its results also serve the error statements)
    mean_mixed, _ = pipeline(Xd, Vd, train, test, wl, "mixed", timings=stages, keep=kept_mixed)
    t_step = replicas.max_over_ranks(t_step, device="cuda")
    out = {}
    if rank == 0:
        # the plain FP64 form of the same step, for the metric's comparison:
        # one untimed run (allocator warm-up), then timed runs (one when a step
        # takes more than ten seconds)
        fp64_times = []
        mean64 = None
        kept64 = {}
        errors = None
        if not args.skip_fp64:
            pipeline(Xd, Vd, train, test, wl, "fp64")
            reps = max(1, min(args.steps, 2))
            for r in range(reps):
                flush_l2(flush)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                mean64, _ = pipeline(Xd, Vd, train, test, wl, "fp64", keep=kept64)
                e1.record(stream)
                torch.cuda.synchronize()
                fp64_times.append(e0.elapsed_time(e1) / 1e3)
                if fp64_times[-1] > 10.0:
                    break
            errors = error_statements(kept_mixed, kept64, mean_mixed, mean64)
            kept64.clear()
        kept_mixed.clear()
        # end to end through the public API with host buffers
        e2e_times = []
        mean_h = var_h = np.zeros(0)
        for _ in range(0 if args.skip_e2e else 2):
            import rvgp_gb300 as RVGP
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Xh = X
            if "n_raw" in wl:  # the public furthest-point sampling on the host array
                from rvgp_gb300.geometry import furthest_point_sampling
                perm_h, _ = furthest_point_sampling(X, N=wl["n"])
                Xh = X[perm_h]
            d = RVGP.create_data_object(Xh, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False, **dim_kwargs(wl))
            d.vectors = V
            gp = RVGP.fit(d, train_ind=train, epochs=wl["adam"], optimizer="adam", lr=0.05, verbose=False)
            mean_h, var_h = gp.transform(d, test)
            d.wait()  # the concurrent eigensolve of L belongs to the step
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
        peaks, src = measured_peaks()
        Xs = sample_points(Xd, wl)  # the points the pipeline runs on
        d = __import__("rvgp_gb300").create_data_object(Xs, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False,
                                                        **dim_kwargs(wl))
        d.wait()  # its L eigensolve runs on a host thread of its own: not beside the timed launches
        torch.cuda.synchronize()
        roof = spmm_roofline(d, wl, peaks, flush)
        d.wait()
        del d
        roof["peak_source"] = src
        pred_err = errors["posterior_mean_rel_err"] if errors else None
        out = {
            "metric": METRIC, "value": round(t_step, 5), "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": bench_config(wl, args, world),
            "fp64_form_s": round(float(np.mean(fp64_times)), 5) if fp64_times else None,
            "mixed_speedup_vs_fp64": round(float(np.mean(fp64_times)) / t_step, 3) if fp64_times else None,
            "pred_rel_err_vs_fp64": pred_err,
            "errors_vs_fp64": errors,
            "pipelines_per_s": round(replicas.job_throughput(t_step, world), 4),
            "stages_s": {k_: (round(v, 5) if isinstance(v, float) else v) for k_, v in stages.items()},
            "e2e": {"value": round(float(np.mean(e2e_times)), 5) if e2e_times else None, "unit": "s",
                    "h2d_bytes_per_step": int(X.nbytes + V.nbytes),
                    "d2h_bytes_per_step": int(mean_h.nbytes + var_h.nbytes)},
            "roofline": roof,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "step_times_s": [round(t, 5) for t in times],
        }
        if not args.skip_cpu:
            # bounded sample (about half a minute of host work): kNN on a share of
            # the queries, the SVDs of a share of the points, capped eigsh, the
            # dense GP at a few thousand rows; the later stages start from this
            # step's graph and gauges
            d_in = __import__("rvgp_gb300").create_data_object(Xs, n_neighbors=wl["k"], n_eigenpairs=wl["m"],
                                                               verbose=False, **dim_kwargs(wl))
            inputs = gpu_inputs(d_in)
            d_in.wait()
            del d_in
            small = wl["n"] > 50000
            out["cpu_baseline"] = cpu_baseline(
                wl, Xs.cpu().numpy(), V, train, test, inputs=inputs,
                caps=dict(eigsh=args.cpu_eigsh_cap / 6, knn_rows=5000 if small else None,
                          frame_rows=10000 if small else None, gp_rows=8192))
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return out


# ------------------------------------------------------------------------------ CPU baseline (oracle port)
def _eigsh_child(path, m, out):
    """Child process of the capped ARPACK timing: eigsh(which='SM') of the
    matrix saved at `path` (RVGP/geometry.py:66-80); writes its wall time."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    z = np.load(path)
    M = sp.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
    t0 = time.perf_counter()
    spla.eigsh(M, k=m, which="SM")
    with open(out, "w") as f:
        f.write(str(time.perf_counter() - t0))


def eigsh_capped(M, m, cap_s):
    """Wall seconds of the reference's eigsh(which='SM') on M, run in a child
    process that is stopped after cap_s: (seconds, finished).  Unfinished runs
    give a lower bound."""
    import multiprocessing as mp
    import tempfile
    M = M.tocsr()
    with tempfile.TemporaryDirectory() as tmp:
        path, out = os.path.join(tmp, "M.npz"), os.path.join(tmp, "t.txt")
        np.savez(path, data=M.data, indices=M.indices, indptr=M.indptr, shape=np.array(M.shape))
        ctx = mp.get_context("spawn")
        p = ctx.Process(target=_eigsh_child, args=(path, m, out))
        t0 = time.perf_counter()
        p.start()
        p.join(cap_s)
        if p.is_alive():
            p.terminate()
            p.join()
            return time.perf_counter() - t0, False
        if os.path.exists(out):
            with open(out) as f:
                return float(f.read()), True
        return time.perf_counter() - t0, False


def cpu_pipeline(wl, X, V, train, test, inputs=None, caps=None):
    """The reference algorithm's stages on the host cores (the oracle's CPU
    restatement: sklearn's brute-force / KD-tree kNN, the heap Dijkstra in C,
    LAPACK SVDs, connections, Laplacians, ARPACK eigsh(which='SM'), GPflow's
    dense GPR likelihood, gradient and predict), each on the full workload or a
    bounded sample of it.  Returns {stage: {"s": seconds for the full workload,
    "measured_s": seconds actually spent, "how": "measured" | "extrapolated"
    | "lower bound", "sample": ...}}.

    ``inputs`` (optional: indptr, indices, gauges T (n, D, d), L values, Lc
    values of the same workload) let the stages after kNN start from the given
    graph and gauges, so that each stage can be sampled on its own; without
    them every stage computes its own inputs on the host.  ``caps``: seconds
    allowed per eigsh (capped runs are lower bounds), rows of the sampled kNN
    queries / tangent frames, and the most training rows the dense GP is
    timed at."""
    from oracle import rvgp_oracle as O
    O.build_c()
    caps = dict(dict(eigsh=60.0, knn_rows=None, frame_rows=None, gp_rows=16384), **(caps or {}))
    n, D = X.shape
    k, m = wl["k"], wl["m"]
    K = int(k * 1.5)
    d = wl.get("dim", 2)
    st = {}

    def put(name, s, measured, how, sample):
        st[name] = {"s": round(s, 3), "measured_s": round(measured, 3), "how": how, "sample": sample}

    # kNN graph (RVGP/geometry.py:100-123)
    rows = caps["knn_rows"]
    t0 = time.perf_counter()
    if D > 15:
        nn = O.knn_gemm(X, k, rows=None if rows is None else np.arange(min(rows, n)))
    else:
        nn = O.knn_kdtree(X, k)
        rows = None
    t = time.perf_counter() - t0
    if rows is None or rows >= n:
        ip, ix = O.symmetrised_csr(nn, n)
        put("graph", time.perf_counter() - t0, time.perf_counter() - t0, "measured",
            "brute force (matrix-product distances)" if D > 15 else "KD-tree")
    else:
        put("graph", t * n / rows, t, "extrapolated", f"{rows} of {n} query rows, linear in the queries")
        ip, ix = inputs["indptr"], inputs["indices"]
    # gauges: geodesic neighbourhoods + local SVDs (RVGP/lib/ptu_dijkstra.pyx:33-125)
    t0 = time.perf_counter()
    nbh = O.geodesic_neighbourhoods(ip, ix, K)
    t_nbh = time.perf_counter() - t0
    fr = caps["frame_rows"]
    t0 = time.perf_counter()
    if fr is None or fr >= n:
        Tg, _ = O.tangent_frames(X, nbh, d)
        t_fr = time.perf_counter() - t0
        put("gauges", t_nbh + t_fr, t_nbh + t_fr, "measured", "every point")
    else:
        O.tangent_frames(X, nbh[:fr], d)
        t_fr = time.perf_counter() - t0
        put("gauges", t_nbh + t_fr * n / fr, t_nbh + t_fr, "extrapolated",
            f"neighbourhoods of every point; SVDs of {fr} of {n} points, linear in the points")
        Tg = inputs["T"][:, :, :d]
    # connections and Laplacians (pyx:128-293, RVGP/geometry.py:14-63)
    t0 = time.perf_counter()
    R = O.connections(np.ascontiguousarray(Tg), ip, ix)
    put("connections", time.perf_counter() - t0, time.perf_counter() - t0, "measured", "every edge")
    t0 = time.perf_counter()
    L = O.laplacian(ip, ix, n)
    Lc = O.connection_laplacian(L, R, ip, ix, d)
    put("laplacians", time.perf_counter() - t0, time.perf_counter() - t0, "measured", "full matrices")
    # eigenpairs (RVGP/geometry.py:66-80): ARPACK, capped
    for name, M in (("eigsh_L", L), ("eigsh_Lc", Lc)):
        t, done = eigsh_capped(M, m, caps["eigsh"])
        put(name, t, t, "measured" if done else "lower bound",
            "eigsh(which='SM') to convergence" if done else
            f"eigsh(which='SM') stopped unconverged after {caps['eigsh']:.0f} s")
    # GP (GPflow GPR, RVGP/main.py:55-95): the dense N x N algebra.  One
    # likelihood + gradient evaluation is timed at the workload's N training
    # rows when N <= gp_rows, and multiplied by the optimiser steps; above
    # that it is timed at N1 = gp_rows / 2 and N2 = gp_rows rows and the cost
    # t(N) = a N² + b N³ (kernel assembly and solves, Cholesky) fitted to
    # the two points is evaluated at N.  Predict likewise, with its N²·T
    # triangular solves linear in the T test rows.
    from oracle.rvgp_oracle import train_test_split_indices
    tr, _ = train_test_split_indices(len(train), 0.2, 0)
    N = len(tr) * D
    Nte = len(test) * D
    rng = np.random.default_rng(0)
    S = O.eval_S(np.linspace(0.0, 1.0, m), 1.5, 5.0, 1.0, float(n * D))
    q = min(Nte, 2000)
    Pte = rng.standard_normal((q, m)) / np.sqrt(m)

    def timed(rows):
        Phi = rng.standard_normal((rows, m)) / np.sqrt(m)
        y = rng.standard_normal(rows)
        t0 = time.perf_counter()
        O.lml_dense(Phi, y, S, 1.0)
        O.lml_grad_S_noise(Phi, y, S, 1.0)
        t_fit = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.predict_f(Phi, y, S, 1.0, Pte)
        return t_fit, time.perf_counter() - t0

    def cubic_fit(N1, t1, N2, t2):
        b = max(0.0, (t2 - (N2 / N1) ** 2 * t1) / (N2 ** 3 - N2 ** 2 * N1))
        a = max(0.0, (t1 - b * N1 ** 3) / N1 ** 2)
        return a, b

    G = caps["gp_rows"]
    if N <= G:
        f, p_ = timed(N)
        put("gp_fit", f * wl["adam"], f, "extrapolated",
            f"one dense LML + gradient evaluation at the workload's {N} rows ({f:.2f} s) x {wl['adam']} "
            f"optimiser steps")
        put("gp_predict", p_ * Nte / q, p_, "extrapolated" if q < Nte else "measured",
            f"dense predict at {N} training rows for {q} of {Nte} test rows, linear in the test rows")
    else:
        N1, N2 = G // 2, G
        f1, p1 = timed(N1)
        f2, p2 = timed(N2)
        a, b = cubic_fit(N1, f1, N2, f2)
        one = a * N * N + b * N ** 3
        put("gp_fit", one * wl["adam"], f1 + f2, "extrapolated",
            f"dense LML + gradient timed at {N1} and {N2} rows ({f1:.2f} s, {f2:.2f} s); t(N) = aN² + bN³ "
            f"fitted to them, at N = {N} rows, x {wl['adam']} optimiser steps; K_y alone needs "
            f"{8.0 * N * N / 1e12:.1f} TB")
        a, b = cubic_fit(N1, p1, N2, p2)
        put("gp_predict", b * N ** 3 + a * N * N * Nte / q, p1 + p2, "extrapolated",
            f"dense predict timed at {N1} and {N2} training rows for {q} test rows; t = bN³ + aN²·T/{q} "
            f"fitted to them, at N = {N}, T = {Nte}")
    return st


def cpu_baseline(wl, X, V, train, test, inputs=None, caps=None):
    t0 = time.perf_counter()
    st = cpu_pipeline(wl, X, V, train, test, inputs=inputs, caps=caps)
    wall = time.perf_counter() - t0
    total = sum(v["s"] for v in st.values())
    hows = {v["how"] for v in st.values()}
    return {"value": round(total, 3), "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "extrapolated": "extrapolated" in hows, "lower_bound_stages": sorted(k_ for k_, v in st.items()
                                                                                if v["how"] == "lower bound"),
            "measured_s": round(sum(v["measured_s"] for v in st.values()), 2), "wall_s": round(wall, 2),
            "sample": ("each stage of the reference algorithm on the full workload or a bounded sample of it "
                       "(per stage: 'how' and 'sample'); 'value' adds the per-stage figures"),
            "stages": st}


def gpu_inputs(d):
    """Graph, gauges and Laplacian values of a data object, as host arrays
    (the inputs the sampled CPU stages start from)."""
    dev = d._dev
    return {"indptr": dev.indptr.cpu().numpy(), "indices": dev.indices.cpu().numpy(), "T": dev.T.cpu().numpy()}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    X, train, test = make_inputs(wl, seed=0)
    rng = np.random.default_rng(0)
    V = rng.standard_normal(X.shape)  # the CPU timing does not depend on the field values
    from oracle import rvgp_oracle as O
    O.build_c()
    for _ in range(args.warmup):  # warm-up: the library loads and a small product
        O.knn_gemm(X[:2000], wl["k"]) if X.shape[1] > 15 else O.knn_kdtree(X[:2000], wl["k"])
    base = cpu_baseline(wl, X, V, train, test, caps=dict(eigsh=args.cpu_eigsh_cap))
    out = {"metric": METRIC, "value": base["value"], "unit": "s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(base["value"] * 1e3, 1),
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": bench_config(wl, args, int(os.environ.get("WORLD_SIZE", "1"))),
           "impl": "reference", "cpu_baseline": base,
           "note": ("one pass of the reference algorithm per invocation (its stages cannot repeat --steps times "
                    "within minutes); stages the host cannot finish are projected or bounded below, each labelled"),
           "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------ sparse GP (--model sgpr)
SGPR_METRIC = "RVGP sparse-GP fit+predict wall s (FPS inducing rows, L-BFGS-B on kernel, noise and Z)"
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (CUDA cores), nominal: no measured FP64 peak exists for this machine


def sgpr_flops(m, M):
    """Algorithmic FP64 flops of one rvgp_sgpr_elbo call with ∂F/∂Z and the
    posterior state: its matrix products (2 r c k each), two Cholesky
    factorisations and two triangular inverses (M³/3 each); vector products
    are left out."""
    g = lambda r, c, k: 2.0 * r * c * k  # noqa: E731
    f = g(M, M, m) + g(M, m, M) + g(M, m, m) + g(M, M, m)          # Kuu, L⁻¹Z, W C, Q0
    f += 4 * M ** 3 / 3.0                                             # chol + inverse of Kuu and B
    f += g(M, m, M) + g(M, m, m) + g(M, M, m) + g(m, M, M)            # V, V C, W Hᵀ, Ẑᵀ(W Hᵀ)
    f += g(m, m, M) + g(M, m, m) + g(m, m, M) + g(M, m, M) + g(M, m, m)  # WᵀW, H Q, HᵀHQ, L⁻ᵀW, ∂F/∂Z
    f += g(m, m, M)                                                   # VᵀV
    return f


def run_sgpr(args):
    import torch
    import rvgp_gb300 as RVGP
    from rvgp_gb300 import _core
    _core.require_cuda()
    wl = WORKLOADS[args.workload]
    M, iters = args.inducing, args.sgpr_iters
    X, train, test = make_inputs(wl, seed=0)
    V = make_field(X, wl, seed=0)
    Xd = torch.as_tensor(X, device="cuda")
    d = RVGP.create_data_object(Xd, n_neighbors=wl["k"], n_eigenpairs=wl["m"], precision="mixed", verbose=False)
    d.vectors = V
    d.wait()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    stream = torch.cuda.current_stream()

    def step():
        gp = RVGP.fit(d, train_ind=train, n_inducing_points=M, epochs=iters, verbose=False)
        return gp, gp.predict_points(test)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times, evals = [], []
    launches0 = _core.launch_count()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gp, (mean, var) = step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            evals.append(gp.n_evals)
    launches = _core.launch_count() - launches0
    t_step = float(np.mean(times))
    # one bound evaluation (with ∂F/∂Z and the posterior) timed alone, L2 flushed before each
    Z = gp.inducing_variable.Z
    th = gp.theta()
    ev_t = []
    torch.cuda.nvtx.range_push("sgpr_eval")  # lets a profiler select exactly these launches
    for r in range(23):
        flush_l2(flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _core.sgpr_elbo(gp.C, gp.b, gp.yy, gp.N, Z, gp.kernel.eigenvalues, gp.kernel.num_verticies, th,
                        gp.kernel.typ, gp.jitter, gp.work)
        e1.record(stream)
        torch.cuda.synchronize()
        if r >= 3:
            ev_t.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.nvtx.range_pop()
    t_eval = float(np.mean(ev_t))
    flops = sgpr_flops(gp.m, M)
    achieved = flops / t_eval / 1e12
    # end to end through the public API with host buffers
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.vectors = V
        g2 = RVGP.fit(d, train_ind=train, n_inducing_points=M, epochs=iters, verbose=False)
        mh, vh = g2.transform(d, test)
        e2e.append(time.perf_counter() - t0)
    out = {
        "metric": SGPR_METRIC, "value": round(t_step, 5), "unit": "s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "model": "manifold_SGPR", "inducing": M, "lbfgsb_max_iter": iters,
                   "N_train_rows": int(gp.N), "m": int(gp.m), "l2": "flushed between steps (256 MiB write)",
                   "step": "fit (FPS, C/b/yᵀy, L-BFGS-B) + predict at the test points; data object built before"},
        "bound_evals_per_step": [int(e) for e in evals], "elbo": gp.elbo(), "l2_error": getattr(gp, "l2_error", None),
        "eval_ms": round(t_eval * 1e3, 4),
        "roofline": {"kernel": "rvgp_sgpr_elbo chain (one bound + gradients + posterior)", "bound": "fp64",
                     "achieved": round(achieved, 4), "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                     "frac": round(achieved / FP64_NOMINAL_TFLOPS, 4), "traffic": None,
                     "peak_source": "nominal", "algorithmic_flops": flops},
        "e2e": {"value": round(float(np.mean(e2e)), 5), "unit": "s", "h2d_bytes_per_step": int(V.nbytes),
                "d2h_bytes_per_step": int(mh.nbytes + vh.nbytes)},
        "clocks": clk.summary(), "gpu_launches": int(launches / max(1, args.steps)),
        "step_times_s": [round(t, 5) for t in times],
    }
    if not args.skip_cpu:
        from oracle import rvgp_oracle as O
        n, m = d.n, gp.m
        ev = d.evecs_Lc.reshape(n, -1)
        tr, _ = O.train_test_split_indices(len(train), 0.2, 0)
        Phi = ev[train[tr]].reshape(-1, m)
        y = V[train[tr]].reshape(-1)
        Zh = Z.cpu().numpy()
        S = O.eval_S(d.evals_Lc, float(gp.kernel.nu), float(gp.kernel.kappa), float(gp.kernel.sigma_f),
                     d.evecs_Lc.shape[0])
        noise = float(gp.likelihood.variance)
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            O.sgpr_elbo(Phi, y, S, noise, Zh)
        one = (time.perf_counter() - t0) / reps
        Phi_te = ev[test].reshape(-1, m)
        sample = min(len(Phi_te), 2000)
        t0 = time.perf_counter()
        O.sgpr_predict_f(Phi, y, S, noise, Zh, Phi_te[:sample])
        t_pred = (time.perf_counter() - t0) * len(Phi_te) / sample
        n_ev = float(np.mean(evals))
        out["cpu_baseline"] = {
            "value": round(one * n_ev + t_pred, 3), "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "sample": (f"GPflow's SGPR bound (value only, no gradient) evaluated {reps}x on the full training rows "
                       f"({one:.3f} s each) and scaled by the {n_ev:.0f} bound evaluations per fit, plus predict "
                       f"on {sample} test rows scaled to all {len(Phi_te)}")}
    print(json.dumps(out), flush=True)
    return out


# ------------------------------------------------------------------------------ RBF GP and field features
RBF_METRIC = "RVGP kernel='rbf' GP fit+predict wall s (scalar eigenbasis, L-BFGS-B on variance, lengthscale, noise)"
FEATURES_METRIC = "vector-field div/curl features: (field, point) pairs per s"


def run_rbf(args):
    """The RBF-kernel GP (fit(kernel='rbf')) on the sphere workload: n = 2000,
    k = 10, 50 eigenpairs, 50 % train (800 training rows after the internal
    split), L-BFGS-B for --sgpr-iters iterations, predict at the other 1000 points."""
    import torch
    import rvgp_gb300 as RVGP
    from rvgp_gb300 import _core
    _core.require_cuda()
    wl = WORKLOADS["sphere_n2000_k10_m50"]
    X, train, test = make_inputs(wl, seed=0)
    d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], precision="fp64", verbose=False)
    d.random_vector_field(seed=0)
    d.smooth_vector_field(t=wl["t_smooth"])
    V = d.vectors
    d.wait()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        gp = RVGP.fit(d, train_ind=train, kernel="rbf", epochs=args.sgpr_iters, verbose=False)
        return gp, gp.predict_points(test)

    for _ in range(args.warmup):
        step()
    times, evals = [], []
    launches0 = _core.launch_count()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gp, _ = step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            evals.append(gp.n_evals)
    launches = _core.launch_count() - launches0
    t_step = float(np.mean(times))
    ev_t = []
    for r in range(13):
        flush_l2(flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _core.rbf_lml(gp.X, gp.Y, gp.theta(), gp.work)
        e1.record(stream)
        torch.cuda.synchronize()
        if r >= 3:
            ev_t.append(e0.elapsed_time(e1) / 1e3)
    t_eval = float(np.mean(ev_t))
    N, m, D = gp.N, gp.m, gp.D
    flops = N ** 3 / 3.0 + N ** 3 / 3.0 + 2.0 * N ** 3 + 3.0 * N * N * m + 4.0 * N * N * D  # chol, L⁻¹, K⁻¹, K, products
    achieved = flops / t_eval / 1e12
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.vectors = V
        g2 = RVGP.fit(d, train_ind=train, kernel="rbf", epochs=args.sgpr_iters, verbose=False)
        mh, vh = g2.transform(d, test)
        e2e.append(time.perf_counter() - t0)
    out = {"metric": RBF_METRIC, "value": round(t_step, 5), "unit": "s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "sphere_n2000_k10_m50", "model": "rbf_GPR", "N_train_rows": int(N), "m": int(m),
                      "outputs": int(D), "lbfgsb_max_iter": args.sgpr_iters, "l2": "flushed between steps"},
           "lml_evals_per_step": [int(e) for e in evals], "l2_error": getattr(gp, "l2_error", None),
           "eval_ms": round(t_eval * 1e3, 4),
           "roofline": {"kernel": "rvgp_rbf_lml chain (likelihood + gradient + posterior state)", "bound": "fp64",
                        "achieved": round(achieved, 4), "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                        "frac": round(achieved / FP64_NOMINAL_TFLOPS, 4), "traffic": None, "peak_source": "nominal",
                        "algorithmic_flops": flops},
           "e2e": {"value": round(float(np.mean(e2e)), 5), "unit": "s", "h2d_bytes_per_step": int(V.nbytes),
                   "d2h_bytes_per_step": int(mh.nbytes + vh.nbytes)},
           "clocks": clk.summary(), "gpu_launches": int(launches / max(1, args.steps)),
           "step_times_s": [round(t, 5) for t in times]}
    if not args.skip_cpu:
        from oracle import rvgp_oracle as O
        Xh, Yh = gp.X.cpu().numpy(), gp.Y.cpu().numpy()
        th = [float(p) for p in gp._slots()]
        t0 = time.perf_counter()
        for _ in range(3):
            O.rbf_gpr_lml(Xh, Yh, *th)
            Ky = O.rbf_K(Xh, Xh, th[0], th[1]) + th[2] * np.eye(N)
            np.linalg.inv(Ky)  # the gradient's K_y⁻¹
        one = (time.perf_counter() - t0) / 3
        t0 = time.perf_counter()
        O.rbf_gpr_predict_f(Xh, Yh, *th, d.evecs_L[test])
        t_pred = time.perf_counter() - t0
        n_ev = float(np.mean(evals))
        out["cpu_baseline"] = {"value": round(one * n_ev + t_pred, 3), "unit": "s", "cores": os.cpu_count(),
                               "kind": "port",
                               "sample": (f"GPflow's GPR likelihood with the RBF kernel plus the K_y⁻¹ of its "
                                          f"gradient, 3x ({one * 1e3:.1f} ms each), scaled by {n_ev:.0f} "
                                          f"evaluations per fit, plus the predict")}
    print(json.dumps(out), flush=True)
    return out


def run_features(args):
    """div/curl features of B = 1024 time samples of a field on n = 20000 torus
    points, k = 5, in one launch per step (compute_vectorfield_features_time)."""
    import torch
    from rvgp_gb300 import _core
    from rvgp_gb300.features import compute_vectorfield_features_time
    _core.require_cuda()
    wl = WORKLOADS["torus_n20000_k20_m200"]
    X, _, _ = make_inputs(wl, seed=0)
    n, B, k = X.shape[0], 1024, 5
    rng = np.random.default_rng(0)
    Vh = rng.standard_normal((B, n, 3))
    P = torch.as_tensor(X, device="cuda")
    V = torch.as_tensor(Vh, device="cuda")
    nbr = _core.knn(P, k)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        _core.vectorfield_features(P, V, nbr)
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _core.vectorfield_features(P, V, nbr)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    t = float(np.mean(times))
    alg = B * n * (3 * 8 + 4 * 8) + n * k * 4 + n * 3 * 8  # fields read once, div + curl written, lists, points
    peaks, src = measured_peaks()
    gbs = alg / t / 1e9
    # FP64 flops per (field, point): the unit vector (norm 5, scaling 3, its
    # reciprocal square root 1) and per neighbour Δu (3), Δu·e (6) and Δu×e
    # (12), then the four 1/k scalings; the geometry pass is per point only
    flops = B * n * (9 + 21 * k + 4)
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        div, curl = compute_vectorfield_features_time(range(B), X, Vh, k=k)
        e2e.append(time.perf_counter() - t0)
    out = {"metric": FEATURES_METRIC, "value": round(B * n / t, 1), "unit": "pairs/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 4), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "torus_n20000 points, 1024 fields, k=5", "l2": "flushed between steps; the "
                      "fields (491 MB) exceed L2"},
           "roofline": {"kernel": "rvgp_vectorfield_features (vf_geometry, vf_unit, vf_features_kernel)",
                        "bound": "fp64", "achieved": round(flops / t / 1e12, 4), "peak": FP64_NOMINAL_TFLOPS,
                        "unit": "TFLOP/s", "frac": round(flops / t / 1e12 / FP64_NOMINAL_TFLOPS, 4),
                        "traffic": None, "peak_source": "nominal", "algorithmic_flops": int(flops),
                        "hbm": {"achieved_gbs": round(gbs, 1), "peak_gbs": peaks["hbm_gbs"],
                                "frac": round(gbs / peaks["hbm_gbs"], 4), "peak_source": src,
                                "algorithmic_bytes": int(alg)}},
           "e2e": {"value": round(B * n / float(np.mean(e2e)), 1), "unit": "pairs/s",
                   "h2d_bytes_per_step": int(Vh.nbytes + X.nbytes), "d2h_bytes_per_step": int(div.nbytes + curl.nbytes)},
           "clocks": clk.summary(), "gpu_launches": 3, "step_times_s": [round(x, 6) for x in times]}
    if not args.skip_cpu:
        from oracle import rvgp_oracle as O
        s = 16
        t0 = time.perf_counter()
        for b in range(s):
            O.vectorfield_features(X, Vh[b], k=k, kdtree=True)
        tc = (time.perf_counter() - t0) / s
        out["cpu_baseline"] = {"value": round(n / tc, 1), "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": (f"the oracle (vectorised numpy, a KD-tree per field as the reference "
                                          f"queries one per call) on {s} of the fields")}
    print(json.dumps(out), flush=True)
    return out


FIELDS_METRIC = ("many fields at shared training points: fields per s (16 hyperparameter restarts + all posteriors, one "
                 "CUDA-graph replay)")


def make_fields(d, B, seed=0, t_range=(20.0, 200.0), noise=0.05):
    """B smoothed random tangent fields on the data object's manifold (input
    generation, untimed): per field a random local vector per point, diffused
    by exp(-t Lc) with t ~ U[t_range] in the spectral form on the computed
    eigenbasis, lifted to ambient coordinates, plus N(0, noise²) noise.
    Returns (B, n, D) on the device."""
    import torch
    dev = d._dev
    g = torch.Generator(device="cuda").manual_seed(seed)
    U = dev.evecs_Lc_local / torch.linalg.vector_norm(dev.evecs_Lc_local, dim=0)
    lam = dev.evals_Lc
    n, D, dm = d.n, dev.X.shape[1], d.dim_man
    t = torch.empty(B, dtype=torch.float64, device="cuda").uniform_(*t_range, generator=g)
    x = torch.randn((U.shape[0], B), dtype=torch.float64, device="cuda", generator=g)
    c = (U.T @ x) * torch.exp(-lam[:, None] * t[None, :])
    loc = (U @ c).reshape(n, dm, B)
    loc = loc / loc.pow(2).sum(1, keepdim=True).mean().sqrt()
    v = torch.einsum("iaq,iqb->bia", dev.T[:, :, :dm], loc)
    return v + noise * torch.randn(v.shape, dtype=torch.float64, device="cuda", generator=g)


def run_fields(args):
    """Many fields at the same training points (the batched multi-RHS
    configuration): upper half ellipsoid (1.0, 0.85, 1.1), n = 10000, k = 12,
    300 eigenpairs, 64 seeded training points, B = 4096 smoothed random
    tangent fields.  One step = one replay of a CUDA graph holding 16 restarts
    (log-uniform initial lengthscales in [0.5, 50]) of the 200-step Adam fit on
    field 0, the best fit's FP64 posterior state, and the posterior means and
    log marginal likelihoods of all 4096 fields at the other 9936 points."""
    import torch
    import rvgp_gb300 as RVGP
    from rvgp_gb300 import _core
    from rvgp_gb300.main import ManyFieldsSolve
    from rvgp_gb300.workloads import make_points
    _core.require_cuda()
    n, k, m, B, n_train, R, epochs = 10000, 12, 300, 4096, 64, 16, 200
    X = make_points("half_ellipsoid", n, seed=0)
    rng = np.random.default_rng(0)
    train = np.sort(rng.choice(n, n_train, replace=False))
    test = np.setdiff1d(np.arange(n), train)
    d = RVGP.create_data_object(X, n_neighbors=k, n_eigenpairs=m, verbose=False)
    fields = make_fields(d, B, seed=1)
    d.vectors = fields[0]
    gp = RVGP.fit(d, train_ind=train, epochs=0, verbose=False)  # rows and C, b, yᵀy of field 0
    starts = gp.restart_starts(R, seed=2)
    solve = ManyFieldsSolve(gp, fields, test, starts, epochs=epochs)
    solve.enqueue()  # eager run: sets every kernel and buffer up
    torch.cuda.synchronize()
    eager_mean = solve.mean.clone()
    solve.capture()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        solve.replay()
    torch.cuda.synchronize()
    replay_err = float((solve.mean - eager_mean).abs().max() / eager_mean.abs().max())
    launches0 = _core.launch_count()
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solve.replay()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    t = float(np.mean(times))
    # eager (no graph) for comparison, and the posterior part alone
    eager = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solve.enqueue()
        e1.record(stream)
        torch.cuda.synchronize()
        eager.append(e0.elapsed_time(e1) / 1e3)
    post = []
    for p, v in zip(gp._slots(), solve.fit["theta_best"].cpu().numpy()):
        if p is not None:
            p.assign(float(v))
    for _ in range(3):
        flush_l2(flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gp.predict_fields(fields, test)
        e1.record(stream)
        torch.cuda.synchronize()
        post.append(e0.elapsed_time(e1) / 1e3)
    t_post = float(np.mean(post))
    N, Nte = gp.N, len(test) * 3
    flops = 2.0 * (N * m * B + 2 * m * m * B + Nte * m * B)
    achieved = flops / t_post / 1e12
    # end to end through the public API with host buffers (fields in, means out)
    fh = fields.cpu().numpy()
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = ManyFieldsSolve(gp, fh, test, starts, epochs=epochs)
        s2.enqueue()
        mh = s2.means().cpu().numpy()
        e2e.append(time.perf_counter() - t0)
    lml = solve.fit["lml"].cpu().numpy()
    out = {"metric": FIELDS_METRIC, "value": round(B / t, 1), "unit": "fields/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (smoothed random tangent fields + noise)",
           "config": {"workload": "half_ellipsoid_n10000_k12_m300", "fields": B, "restarts": R, "adam_steps": epochs,
                      "train_points": n_train, "test_points": int(len(test)),
                      "l2": "flushed between steps; the means (976 MB) exceed L2"},
           "step": "one CUDA-graph replay: 16 restarts of the fit + FP64 state + posterior of every field",
           "graph_replay_s": round(t, 5), "eager_s": round(float(np.mean(eager)), 5),
           "replay_vs_eager_max_rel_diff": replay_err, "posterior_only_s": round(t_post, 5),
           "restart_lml": [round(float(v), 3) for v in lml], "best_restart": int(solve.fit["best"].cpu().numpy()[0]),
           "roofline": {"kernel": "rvgp_gp_posterior_batch (FP64 products)", "bound": "fp64",
                        "achieved": round(achieved, 4), "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                        "frac": round(achieved / FP64_NOMINAL_TFLOPS, 4), "traffic": None, "peak_source": "nominal",
                        "algorithmic_flops": flops},
           "e2e": {"value": round(B / float(np.mean(e2e)), 1), "unit": "fields/s", "h2d_bytes_per_step": int(fh.nbytes),
                   "d2h_bytes_per_step": int(mh.nbytes)},
           "clocks": clk.summary(), "gpu_launches": int((_core.launch_count() - launches0)),
           "step_times_s": [round(x, 5) for x in times]}
    if not args.skip_cpu:
        from oracle import rvgp_oracle as O
        ev = d.evecs_Lc.reshape(n, -1)
        tr, _ = O.train_test_split_indices(len(train), 0.2, 0)
        Phi = ev[train[tr]].reshape(-1, m)
        S = O.eval_S(d.evals_Lc, float(gp.kernel.nu), float(gp.kernel.kappa), float(gp.kernel.sigma_f),
                     d.evecs_Lc.shape[0])
        Ps = ev[test].reshape(-1, m)
        s_ = 4
        t0 = time.perf_counter()
        for b_ in range(s_):
            O.predict_f_lowrank(Phi, fh[b_][train[tr]].reshape(-1), S, float(gp.likelihood.variance), Ps)
        tc = (time.perf_counter() - t0) / s_
        yv = fh[0][train[tr]].reshape(-1)
        t0 = time.perf_counter()
        O.lml_dense(Phi, yv, S, 1.0)
        O.lml_grad_S_noise(Phi, yv, S, 1.0)
        te = time.perf_counter() - t0
        total = tc * B + te * epochs * R
        out["cpu_baseline"] = {"value": round(B / total, 3), "unit": "fields/s", "cores": os.cpu_count(),
                               "kind": "port", "extrapolated": True,
                               "sample": (f"the oracle's posterior per field timed on {s_} fields ({tc:.4f} s each) x "
                                          f"{B}, plus one dense LML + gradient of field 0 ({te:.4f} s) x {epochs} "
                                          f"steps x {R} restarts")}
    print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--cpu-eigsh-cap", type=float, default=60.0,
                    help="seconds allowed per ARPACK eigsh in the reference arm (capped runs are lower bounds)")
    ap.add_argument("--model", choices=["gpr", "sgpr", "rbf", "features", "fields"], default="gpr",
                    help="sgpr: the sparse inducing-point GP fit; rbf: the kernel='rbf' GP; features: div/curl")
    ap.add_argument("--inducing", type=int, default=100, help="inducing rows for --model sgpr")
    ap.add_argument("--sgpr-iters", type=int, default=200, help="L-BFGS-B iterations for --model sgpr / rbf")
    args = ap.parse_args()
    if args.model != "gpr" and args.workload == DEFAULT_WORKLOAD:
        args.workload = "torus_n20000_k20_m200"  # the side models' workload
    if args.model != "gpr":
        runner, metric = {"sgpr": (run_sgpr, SGPR_METRIC), "rbf": (run_rbf, RBF_METRIC),
                          "features": (run_features, FEATURES_METRIC), "fields": (run_fields, FIELDS_METRIC)}[args.model]
        if args.impl == "ours" and int(os.environ.get("RANK", "0")) == 0:
            runner(args)
        elif args.impl == "reference":
            print(json.dumps({"impl": "reference", "metric": metric,
                              "unavailable": "this model's CPU baseline is the cpu_baseline of the ours arm"}))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
