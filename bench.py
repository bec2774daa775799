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
    "torus_n20000_k20_m200": dict(kind="torus", n=20000, k=20, m=200, train_frac=0.3, t_smooth=50.0, adam=200,
                                  rotational=True),
    "sphere_n2000_k10_m50": dict(kind="sphere", n=2000, k=10, m=50, train_frac=0.5, t_smooth=100.0, adam=200,
                                 rotational=False),
}
METRIC = "RVGP fit+predict wall s (mixed vs FP64 GPU, equal pred. error); HBM GB/s"


def make_inputs(wl, seed=0):
    from rvgp_gb300.workloads import make_points, rotational_field, split
    X = make_points(wl["kind"], wl["n"], seed=seed)
    train, test = split(wl["n"], wl["train_frac"], seed=seed)
    return X, train, test


def make_field(X, wl, seed=0):
    """Ground-truth field (outside the timed region): rotational + smoothed random tangent field."""
    import rvgp_gb300 as RVGP
    from rvgp_gb300.workloads import rotational_field
    d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False)
    d.random_vector_field(seed=seed)
    d.smooth_vector_field(t=wl["t_smooth"])
    v = d.vectors
    if wl["rotational"]:
        import torch
        from rvgp_gb300 import _core
        rot = torch.as_tensor(rotational_field(X), device="cuda")
        rot = _core.frame_map(d._dev.T, d.dim_man, rot, "project")
        v = v + rot.cpu().numpy()
    return np.ascontiguousarray(v)


# ------------------------------------------------------------------------------ our arm
def pipeline(X, V, train, test, wl, precision, timings=None):
    """One step through the public API; returns (mean, var) on the device."""
    import torch
    import rvgp_gb300 as RVGP
    d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], precision=precision, verbose=False,
                                timings=timings)
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


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of an ncu capture of
# the launches timed below (Morton-renumbered Lc, torus n=20000, k=20, p=228, L2
# flushed before each) on GB300: 82.34 MB read (exactly the algorithmic reads)
# + 10.61 MB written by the end of the launch (the rest of Y is still in L2).
SPMM_TRAFFIC_BYTES = 92_953_088


def spmm_roofline(d, wl, peaks, flush, reps=20):
    """Achieved HBM bandwidth of the eigensolver's Chebyshev-step SpMM (FP32,
    block width p) on this workload's connection Laplacian: each launch timed
    alone with CUDA events on the launching stream, L2 flushed before it.  The
    matrix is the Morton-renumbered one the eigensolver multiplies by."""
    import torch
    from rvgp_gb300 import _core
    dev = d._dev
    ip, ix, _, v32 = _core.permute_csr(dev.indptr, dev.indices, dev.Lc_vals, dev.Lc_vals32, dev.perm, dev.rank)
    n, k = d.n, d.dim_man
    N = n * k
    p = _core.block_size(wl["m"], N)
    torch.cuda.nvtx.range_push("spmm_roofline")  # lets a profiler select exactly these launches
    X = torch.randn((N, p), dtype=torch.float32, device="cuda")
    Z = torch.randn_like(X)
    Y = torch.empty_like(X)
    for _ in range(3):
        _core.bspmm(ip, ix, v32, X, Y, Z, 0.1, -0.2, 0.3)
    s = torch.cuda.current_stream()
    times = []
    for _ in range(reps):
        flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        _core.bspmm(ip, ix, v32, X, Y, Z, 0.1, -0.2, 0.3)
        e1.record(s)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.nvtx.range_pop()
    t = float(np.mean(times))
    E = dev.indices.numel()
    alg = E * (k * k * 4 + 4) + (n + 1) * 4 + 3 * N * p * 4  # values + indices + read X, read Z, write Y
    achieved = alg / t / 1e9
    same_shape = (n, k, p, E) == (20000, 2, 228, 460824)
    return {"kernel": "bspmm_kernel<float,2> (Chebyshev step, Lc x block)", "bound": "hbm",
            "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4),
            "traffic": SPMM_TRAFFIC_BYTES if same_shape else None, "algorithmic_bytes": int(alg),
            "avg_launch_us": round(t * 1e6, 2), "block_width": p, "l2": "flushed before every timed launch"}


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
            mean_mixed, _ = pipeline(Xd, Vd, train, test, wl, "mixed")
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            barrier()
            times.append(e0.elapsed_time(e1) / 1e3)
    launches = _core.launch_count() - launches0
    t_step = float(np.mean(times))
    stages = {}
    pipeline(Xd, Vd, train, test, wl, "mixed", timings=stages)  # untimed step with a per-stage breakdown
    t_step = replicas.max_over_ranks(t_step, device="cuda")
    out = {}
    if rank == 0:
        # the plain FP64 form of the same step, for the metric's comparison
        fp64_times = []
        mean64 = None
        if not args.skip_fp64:
            pipeline(Xd, Vd, train, test, wl, "fp64")
            for _ in range(max(1, min(args.steps, 2))):
                flush_l2(flush)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                mean64, _ = pipeline(Xd, Vd, train, test, wl, "fp64")
                e1.record(stream)
                torch.cuda.synchronize()
                fp64_times.append(e0.elapsed_time(e1) / 1e3)
        # end to end through the public API with host buffers
        e2e_times = []
        mean_h = var_h = np.zeros(0)
        for _ in range(0 if args.skip_e2e else 2):
            import rvgp_gb300 as RVGP
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d = RVGP.create_data_object(X, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False)
            d.vectors = V
            gp = RVGP.fit(d, train_ind=train, epochs=wl["adam"], optimizer="adam", lr=0.05, verbose=False)
            mean_h, var_h = gp.transform(d, test)
            d.wait()  # the concurrent eigensolve of L belongs to the step
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
        peaks, src = measured_peaks()
        d = __import__("rvgp_gb300").create_data_object(Xd, n_neighbors=wl["k"], n_eigenpairs=wl["m"], verbose=False)
        roof = spmm_roofline(d, wl, peaks, flush)
        roof["peak_source"] = src
        pred_err = None
        if mean64 is not None:
            pred_err = float(torch.linalg.vector_norm(mean_mixed - mean64) / torch.linalg.vector_norm(mean64))
        out = {
            "metric": METRIC, "value": round(t_step, 5), "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": args.workload, "n": wl["n"], "D": 3, "k": wl["k"], "m": wl["m"],
                       "train_frac": wl["train_frac"], "adam_steps": wl["adam"], "parallelism": f"replicas{world}",
                       "l2": "flushed between steps (256 MiB write)"},
            "fp64_form_s": round(float(np.mean(fp64_times)), 5) if fp64_times else None,
            "mixed_speedup_vs_fp64": round(float(np.mean(fp64_times)) / t_step, 3) if fp64_times else None,
            "pred_rel_err_vs_fp64": pred_err,
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
            out["cpu_baseline"] = cpu_baseline(wl, X, V, train, test, budget=args.cpu_budget)
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return out


# ------------------------------------------------------------------------------ CPU baseline (oracle port)
def cpu_stage_times(wl, X, V, train, test, budget=240.0):
    """Per-stage seconds of the reference algorithm's CPU restatement (oracle):
    KD-tree kNN, heap Dijkstra gauges, LAPACK SVDs, connections,
    Laplacians, ARPACK eigsh(which='SM') for L and Lc, one dense GPflow-GPR
    LML + gradient evaluation (scaled by the number of optimiser steps) and the
    dense predict."""
    import math
    from oracle import rvgp_oracle as O
    n, k, m = wl["n"], wl["k"], wl["m"]
    T = {}
    t0 = time.perf_counter()
    nn = O.knn_kdtree(X, k)  # tree search, as sklearn's kneighbors_graph does for 3-d points
    ip, ix = O.symmetrised_csr(nn, n)
    T["graph"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    K = int(k * 1.5)
    nbh = O.geodesic_neighbourhoods(ip, ix, K)
    Tg, S = O.tangent_frames(X, nbh, min(3, K + 1))
    T["gauges"] = time.perf_counter() - t0
    d = O.manifold_dimension(S, 0.8)
    Tg = np.ascontiguousarray(Tg[:, :, :d])
    t0 = time.perf_counter()
    R = O.connections(Tg, ip, ix)
    T["connections"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    L = O.laplacian(ip, ix, n)
    Lc = O.connection_laplacian(L, R, ip, ix, d)
    T["laplacians"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.spectrum(L, m)
    T["eigsh_L"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ev, U = O.spectrum(Lc, m)
    T["eigsh_Lc"] = time.perf_counter() - t0
    evecs = O.lift(Tg, U, m)
    tr, te = O.train_test_split_indices(len(train), 0.2, 0)
    pts = train[tr]
    Phi = evecs.reshape(n, -1)[pts].reshape(-1, m)
    y = V[pts].reshape(-1)
    Sk = O.eval_S(ev, 1.5, 5.0, 1.0, evecs.shape[0])
    t0 = time.perf_counter()
    O.lml_dense(Phi, y, Sk, 1.0)
    O.lml_grad_S_noise(Phi, y, Sk, 1.0)
    one = time.perf_counter() - t0
    T["gp_fit"] = one * wl["adam"]
    Phi_te = evecs.reshape(n, -1)[test].reshape(-1, m)
    sample = min(len(Phi_te), 2000)
    t0 = time.perf_counter()
    O.predict_f(Phi, y, Sk, 1.0, Phi_te[:sample])
    T["gp_predict"] = (time.perf_counter() - t0) * len(Phi_te) / sample  # linear in the test rows
    return T, one


def cpu_baseline(wl, X, V, train, test, budget=240.0):
    T, one = cpu_stage_times(wl, X, V, train, test, budget)
    measured = sum(v for k_, v in T.items() if k_ != "gp_fit") + one
    return {"value": round(sum(T.values()), 3), "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "sample": (f"one pass of every stage on the full workload (measured {measured:.1f} s of CPU time); "
                       f"the GP fit is one dense LML+gradient evaluation scaled by {wl['adam']} optimiser steps; "
                       f"the dense predict is timed on 2000 test rows and scaled to all of them"),
            "stages_s": {k_: round(v, 3) for k_, v in T.items()}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    X, train, test = make_inputs(wl, seed=0)
    rng = np.random.default_rng(0)
    V = rng.standard_normal(X.shape)  # the CPU timing does not depend on the field values
    # warm-up steps exercise the cheap stages only; the timed work is one full stage pass
    from oracle import rvgp_oracle as O
    O.build_c()
    for _ in range(args.warmup):
        O.knn(X[:2000], wl["k"])
    t0 = time.perf_counter()
    base = cpu_baseline(wl, X, V, train, test, budget=args.cpu_budget)
    wall = time.perf_counter() - t0
    out = {"metric": METRIC, "value": base["value"], "unit": "s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(base["value"] * 1e3, 1),
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload, "n": wl["n"], "D": 3, "k": wl["k"], "m": wl["m"],
                      "train_frac": wl["train_frac"], "adam_steps": wl["adam"]},
           "impl": "reference", "cpu_baseline": {**base, "wall_s": round(wall, 2)},
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
                        "bound": "hbm", "achieved": round(gbs, 1),
                        "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": round(gbs / peaks["hbm_gbs"], 4),
                        "traffic": None, "peak_source": src, "algorithmic_bytes": int(alg)},
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


FIELDS_METRIC = "posteriors of many fields at shared training points: fields per s"


def run_fields(args):
    """Many fields at the same training points (the batched multi-RHS shape):
    upper half ellipsoid (1.0, 0.85, 1.1), n = 10000, k = 12, 300 eigenpairs,
    64 seeded training points, B = 4096 fields; one step = predict_fields for
    all fields at the other 9936 points with the hyperparameters of a fit on
    field 0.  Field values are seeded normal vectors (the timing does not depend
    on them)."""
    import torch
    import rvgp_gb300 as RVGP
    from rvgp_gb300 import _core
    from rvgp_gb300.workloads import make_points
    _core.require_cuda()
    n, k, m, B, n_train = 10000, 12, 300, 4096, 64
    X = make_points("half_ellipsoid", n, seed=0)
    rng = np.random.default_rng(0)
    train = np.sort(rng.choice(n, n_train, replace=False))
    test = np.setdiff1d(np.arange(n), train)
    d = RVGP.create_data_object(X, n_neighbors=k, n_eigenpairs=m, precision="fp64", verbose=False)
    fields = torch.randn((B, n, 3), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    d.vectors = fields[0]
    gp = RVGP.fit(d, train_ind=train, epochs=args.sgpr_iters, optimizer="adam", lr=0.05, verbose=False)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    launches0 = _core.launch_count()
    for _ in range(args.warmup):
        gp.predict_fields(fields, test)
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            means, lml = gp.predict_fields(fields, test)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    launches = (_core.launch_count() - launches0) // max(1, args.steps + args.warmup)
    t = float(np.mean(times))
    N, Nte = gp.N, len(test) * 3
    flops = 2.0 * (N * m * B + 2 * m * m * B + Nte * m * B)
    achieved = flops / t / 1e12
    fh = fields.cpu().numpy()
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mh, lh = gp.predict_fields(fh, test)
        mh = mh.cpu().numpy()
        e2e.append(time.perf_counter() - t0)
    out = {"metric": FIELDS_METRIC, "value": round(B / t, 1), "unit": "fields/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded normal field values)",
           "config": {"workload": "half_ellipsoid_n10000_k12_m300", "fields": B, "train_points": n_train,
                      "test_points": int(len(test)), "l2": "flushed between steps; the means (976 MB) exceed L2"},
           "roofline": {"kernel": "rvgp_gp_posterior_batch (FP64 products)", "bound": "fp64",
                        "achieved": round(achieved, 4), "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                        "frac": round(achieved / FP64_NOMINAL_TFLOPS, 4), "traffic": None, "peak_source": "nominal",
                        "algorithmic_flops": flops},
           "e2e": {"value": round(B / float(np.mean(e2e)), 1), "unit": "fields/s", "h2d_bytes_per_step": int(fh.nbytes),
                   "d2h_bytes_per_step": int(mh.nbytes)},
           "clocks": clk.summary(), "gpu_launches": int(launches), "step_times_s": [round(x, 5) for x in times]}
    if not args.skip_cpu:
        from oracle import rvgp_oracle as O
        ev = d.evecs_Lc.reshape(n, -1)
        tr, _ = O.train_test_split_indices(len(train), 0.2, 0)
        Phi = ev[train[tr]].reshape(-1, m)
        S = O.eval_S(d.evals_Lc, float(gp.kernel.nu), float(gp.kernel.kappa), float(gp.kernel.sigma_f),
                     d.evecs_Lc.shape[0])
        Ps = ev[test].reshape(-1, m)
        s = 4
        t0 = time.perf_counter()
        for b in range(s):
            O.predict_f_lowrank(Phi, fh[b][train[tr]].reshape(-1), S, float(gp.likelihood.variance), Ps)
        tc = (time.perf_counter() - t0) / s
        out["cpu_baseline"] = {"value": round(1.0 / tc, 2), "unit": "fields/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"the oracle's rank-m posterior, one field at a time, {s} fields"}
    print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="torus_n20000_k20_m200")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=240.0)
    ap.add_argument("--model", choices=["gpr", "sgpr", "rbf", "features", "fields"], default="gpr",
                    help="sgpr: the sparse inducing-point GP fit; rbf: the kernel='rbf' GP; features: div/curl")
    ap.add_argument("--inducing", type=int, default=100, help="inducing rows for --model sgpr")
    ap.add_argument("--sgpr-iters", type=int, default=200, help="L-BFGS-B iterations for --model sgpr / rbf")
    args = ap.parse_args()
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
