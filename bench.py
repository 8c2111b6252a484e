"""Benchmark: wall-RPY M.F throughput (Gpairs/s) on one GB300.

Workload (one "step"): one wall-corrected RPY product u = M_UF F, FP64-accurate,
over the 256-shell suspension (256 bodies x 42 blobs = 10,752 blobs, a = 0.2436,
x,y ~ U[0,60R], z ~ U[1.2R,5R], forces N(0,1), seed 1), with the inputs
resident in HBM.  One step evaluates N^2 = 1.156e8 ordered pairs.  Inputs are
far smaller than L2, so a 512 MB buffer is written between timed steps to
flush L2.

The headline runs the df64 mode: double-float pair arithmetic on the FP32 pipe
with FP64 accumulation, tested to <= 1e-12 relative error against the FP64
oracle (the FP64-mode bar).  GB300's FP64 pipe runs at 1/74 of its FP32 pipe,
so the native-FP64 kernel (reported under "products" as uf_fp64) is 6x slower.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's own CPU algorithm for the same product
(the oracle's restatement of mobility/mobility.cpp:256-430: symmetric pair
loop, OpenMP over all host cores, -O3 -ffast-math) on the same workload.
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

FLOPS_PER_PAIR = {"uf": 200.0, "ut": 115.0, "wf": 115.0, "wt": 125.0}  # counted from the reference source
METRIC = "wall-RPY M.F Gpairs/s"
HEAD_MODE = "df64"
WORKLOAD = "wall-RPY M_UF.F, 256 shells x 42 blobs = 10,752 blobs (FP64-accurate: df64, <= 1e-12 vs FP64)"
# Split of the near-field augmented preconditioner, in body radii R: exact blob-level couplings below
# NF_EXACT_R, learned mode couplings from there to the network's cutoff NF_CUTOFF_R.  A sweep of the 256-,
# 1024- and 4096-shell mixed solves over exact cutoffs 3R-9R and networks of 6R and 9R range gave the
# fewest iterations and the shortest solves overall with exact couplings below 6R and a 9R network;
# NF_ALL_EXACT_R is the comparison arm with exact couplings of every pair the network would cover.
NF_EXACT_R = 6.0
NF_CUTOFF_R = 9.0
NF_ALL_EXACT_R = NF_CUTOFF_R
# Issued thread instructions per ordered pair of the df64 UF kernels (all
# pipes, 80-85 % of them on the FMA pipe), from ncu's smsp__inst_executed.sum
# on the 10,752-blob product: symmetric kernel (each unordered pair once),
# 1,705,420,652 warp instructions * 32 / 10752^2 = 472.1; one-sided kernel
# (source split 15) 2,719,541,740 * 32 / 10752^2 = 752.8.  The FP32 pipe
# issues at most one thread instruction per lane per clock, the rate the
# FMA-chain probe measures (FLOP/s / 2), so achieved / peak is the fraction of
# issue capacity used.  The constants hold for the kernel sources whose hash is
# DF64_UF_KERNEL_SOURCE_SHA (tests/test_bench_constants.py fails when the
# kernel changes without a new capture).
DF64_UF_INST_PER_PAIR = {"symmetric": 1705420652.0 * 32 / 10752 ** 2, "standard": 2719541740.0 * 32 / 10752 ** 2}
# dram__bytes_read.sum + dram__bytes_write.sum per launch, same captures
DF64_UF_TRAFFIC_BYTES = {"symmetric": 736000, "standard": 718848}
# issued thread instructions per pair and right-hand side of the 16-wide multi-RHS M_UF kernel
# (smsp__inst_executed.sum * 32 / (N^2 * 16), 60,000 blobs)
MULTI16_INST_PER_PAIR_RHS = 17.4
DF64_UF_KERNEL_SOURCE_SHA = "89b6f0fd4303f7413dd2bee1784d821e0f30340b3afe8b244a7c7d322d3f7b63"


def df64_uf_kernel_source_sha():
    """SHA-256 of the sources that fix the df64 M_UF kernels' instruction stream: the device part of
    csrc/wall_pair.cu up to the symmetric UF kernel, and the double-float headers it includes."""
    import hashlib
    d = os.path.join(ROOT, "rigidmultiblobswall_gb300", "csrc")
    h = hashlib.sha256()
    with open(os.path.join(d, "wall_pair.cu")) as fh:
        src = fh.read()
    beg = src.index("namespace rmw {")
    end = src.index("// The rotation blocks (UT, WF, WT) on the same grid")
    h.update(src[beg:end].encode())
    for name in ("pair_math_df.cuh", "dfloat.cuh"):
        with open(os.path.join(d, name)) as fh:
            h.update(fh.read().encode())
    with open(os.path.join(d, "rmw_common.cuh")) as fh:
        src = fh.read()
    h.update(src[src.index("// ---- compensated FP32 accumulation"):].encode())
    return h.hexdigest()


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)  # ~1 s timed: several clock samples
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the per-product secondary timings")
    p.add_argument("--cpu-seconds", type=float, default=8.0)
    p.add_argument("--large", action="store_true",
                   help="only run the 4096-shell (172,032-blob) solve comparison and print its JSON line")
    p.add_argument("--large-modes",
                   default="fp64,mixed,mixed+exact,mixed+learned,mixed+learned_band,mixed+exact+learned,mixed+exact_all")
    p.add_argument("--pc-probe", action="store_true",
                   help="only the 4096-shell block-diagonal preconditioner applies (FP64 and FP32), timed")
    p.add_argument("--krylov-probe", action="store_true",
                   help="only the 4096-shell mixed solve with graphs off (each fused Arnoldi step a traced direct "
                        "launch) and the pair scratch capped at 1 GiB: the Arnoldi steps' time and bandwidth")
    p.add_argument("--bd-probe", action="store_true",
                   help="one Brownian step of the 1024 12-blob shells, plain and learned, in NVTX ranges (for ncu)")
    p.add_argument("--lanczos-probe", type=int, nargs="?", const=64, default=None, metavar="NSUSP",
                   help="the 16-RHS Lanczos of the first NSUSP (default 64) uneven suspensions with every step a "
                        "launch of its own (for ncu)")
    p.add_argument("--multi", default=None, metavar="N:NRHS",
                   help="only time the multi-right-hand-side M_UF product on N blobs with NRHS vectors")
    p.add_argument("--product", default=None, metavar="KIND:MODE",
                   help="only time one wall product (kind uf|ut|wf|wt, mode fp64|df64|mixed) on the headline "
                        "workload for --steps steps after --warmup, and print its JSON line")
    return p.parse_args()


def workload():
    from rigidmultiblobswall_gb300 import suspensions as S
    s = S.shells_42_256()
    r = s.r_vectors()
    f = np.random.default_rng(1).standard_normal(r.shape)
    return s, r, f


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return ws, rank


def hbm_peak_gbs():
    """Measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json), else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def arnoldi_traffic(fn):
    """Run fn() with tracing on and CUDA graphs off (the fused Arnoldi step kernels then launch one by one
    and are timed each); return (fn's result, the Arnoldi orthogonalisation's time, algorithmic bytes and
    bandwidth against the HBM peak)."""
    from rigidmultiblobswall_gb300 import _native
    _native.use_graphs(False)
    _native.trace_enable(True)
    _native.trace_read(1, reset=True)
    _native.trace_bytes(1, reset=True)
    res = fn()
    ms, launches = _native.trace_read(1, reset=True)
    nbytes = _native.trace_bytes(1, reset=True)
    for k in (0, 2, 3, 4, 5, 6, 7):
        _native.trace_read(k, reset=True)
    _native.trace_enable(False)
    _native.use_graphs(True)
    peak, src = hbm_peak_gbs()
    gbs = nbytes / (ms * 1e-3) / 1e9 if ms > 0 else None
    return res, {"steps": launches, "ms": ms, "gbytes": nbytes / 1e9, "gbs": gbs,
                 "frac_of_hbm": (gbs / peak) if gbs else None, "hbm_peak_gbs": peak, "peak_source": src,
                 "bytes_per_step": "(4j + 12) n doubles: CGS2 = 2 x (dots + update) + scale",
                 "kernel": "arnoldi_step_kernel (fused CGS2 + Givens, one launch per step)"}


def pc_apply_roofline(sys_, reps=30):
    """Block-diagonal preconditioner apply, FP64 (FP64 and df64 solves) and FP32 (the mixed solves), timed
    with CUDA events over reps applies with the plain preconditioner built.  Bytes: the per-body matrices
    the kernel reads once per apply, M_b^-1 (m^2) and M_b^-1 K (6m) and N_b (36), times the element size,
    plus the input and output vectors (FP64); the survey's unit for the reference's apply (two dense
    GEMVs per body, 2 m^2 + 12 m + 36 elements) is reported beside it."""
    import torch
    m = np.diff(sys_.offsets) * 3
    out = {}
    x = torch.randn(sys_.size, dtype=torch.float64, device=sys_.device,
                    generator=torch.Generator(device=sys_.device).manual_seed(9))
    peak, src = hbm_peak_gbs()
    for mode, es in (("fp64", 8), ("mixed", 4)):
        sys_.apply_pc(x, mode=mode)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            sys_.apply_pc(x, mode=mode)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        nbytes = float(np.sum(m * m + 6 * m + 36)) * es + 2 * 8.0 * sys_.size
        survey = float(np.sum(2 * m * m + 12 * m + 36)) * es
        out[mode] = {"us": ms * 1e3, "bytes": nbytes, "gbs": nbytes / (ms * 1e-3) / 1e9,
                     "frac_of_hbm": nbytes / (ms * 1e-3) / 1e9 / peak, "survey_unit_bytes": survey,
                     "survey_unit_gbs": survey / (ms * 1e-3) / 1e9}
    out["hbm_peak_gbs"], out["peak_source"] = peak, src
    return out


def reduce_step_ms(step_ms, ws, device=None):
    """Max over ranks of the timed-region milliseconds (every rank calls it)."""
    if ws == 1:
        return float(step_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(step_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gpairs(step_ms_max, ws, steps, n):
    """Whole-job pairs per second: every replica evaluates steps x N^2 pairs."""
    return ws * steps * n * n / (step_ms_max * 1e-3) / 1e9


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(r, f, eta, a, seconds):
    """The oracle's restatement of the reference C++ product on all host cores."""
    from oracle import wall
    threads = os.cpu_count() or 1
    wall.uf_symmetric_fast(r[:512], f[:512], eta, a, threads=threads)  # warm-up (thread pool, pages)
    n = len(r)
    times = []
    t_end = time.perf_counter() + seconds
    while len(times) < 3 or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        wall.uf_symmetric_fast(r, f, eta, a, threads=threads)
        times.append(time.perf_counter() - t0)
        if len(times) >= 200:
            break
    med = float(np.median(times))
    return {"value": n * n / med / 1e9, "unit": "Gpairs/s", "cores": threads, "kind": "port",
            "sample": "%d full M_UF.F products at N=%d (median %.3f s each); oracle/wall_oracle.c "
                      "oracle_wall_uf_symmetric, restating mobility/mobility.cpp:256-430 with the reference's flags "
                      "(-O3 -ffast-math, native CPU tuning, -fopenmp)" % (len(times), n, med)}


def run_reference(args):
    ws, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    s, r, f = workload()
    from oracle import wall
    threads = os.cpu_count() or 1
    n = len(r)
    for _ in range(max(args.warmup, 1)):
        wall.uf_symmetric_fast(r, f, s.eta, s.a, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wall.uf_symmetric_fast(r, f, s.eta, s.a, threads=threads)
    dt = time.perf_counter() - t0
    val = args.steps * n * n / dt / 1e9
    line = {"metric": METRIC, "value": val, "unit": "Gpairs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "n_blobs": n, "pairs_per_step": n * n, "l2": "CPU run"},
            "cpu_baseline": {"value": val, "unit": "Gpairs/s", "cores": threads, "kind": "port",
                             "sample": "%d full M_UF.F products at N=%d per timed run; oracle restatement of "
                                       "mobility/mobility.cpp:256-430 (the reference C++ needs Eigen, absent)"
                                       % (args.steps, n)},
            "e2e": {"value": val, "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def time_product(kind, mode, rt, ft, out_fn, eta, a, steps, flush, stream):
    import torch
    from rigidmultiblobswall_gb300 import mobility as mb
    from rigidmultiblobswall_gb300 import _native
    n = rt.shape[0]
    for _ in range(2):
        mb.wall_product(kind, rt, ft, eta, a, mode=mode)
    _native.trace_enable(True)
    _native.trace_read(0, reset=True)
    evs = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mb.wall_product(kind, rt, ft, eta, a, mode=mode)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / steps
    pair_ms, launches = _native.trace_read(0, reset=True)
    _native.trace_enable(False)
    return {"ms": ms, "gpairs": n * n / (ms * 1e-3) / 1e9, "pair_kernel_ms": pair_ms / max(launches, 1)}


def cfg1_metrics(dev, flush, stream, cpu_seconds=2.0):
    """The plain FP64 translational product of 2,048 free blobs (a = 0.5, eta = 1, x,y ~ U[0,64a],
    z ~ U[1.5a,10a], forces N(0,1), seed 0): native FP64 and df64 kernels (CUDA events per product, L2
    flushed between products), the host-buffer drop-in end to end, and the oracle's restatement of the
    reference C++ product on all host cores, on the same inputs."""
    import torch
    from oracle import wall
    from rigidmultiblobswall_gb300 import mobility as mb
    from rigidmultiblobswall_gb300 import suspensions as S
    r, f, eta, a = S.blobs_wall_matvec(2048, seed=0)
    n = len(r)
    rt = torch.tensor(r, device=dev)
    ft = torch.tensor(f, device=dev)
    out = {"workload": "2,048 free blobs, a = 0.5, eta = 1, x,y ~ U[0,64a], z ~ U[1.5a,10a], F ~ N(0,1), seed 0",
           "pairs_per_product": n * n}
    ref = wall.wall_product("uf", r, f.reshape(-1), eta, a)
    for mode in ("fp64", "df64"):
        mb.autotune("uf", n, mode, reps=5)
        res = time_product("uf", mode, rt, ft, None, eta, a, 40, flush, stream)
        u = mb.wall_product("uf", rt, ft, eta, a, mode=mode).cpu().numpy()
        res["rel_err_vs_oracle"] = float(np.linalg.norm(u - ref) / np.linalg.norm(ref))
        out["uf_" + mode] = res
    rp = torch.empty(r.shape, dtype=torch.float64).pin_memory().numpy()
    fp = torch.empty(f.shape, dtype=torch.float64).pin_memory().numpy()
    rp[:] = r
    fp[:] = f
    for mode in ("fp64", "df64"):
        mb.single_wall_mobility_trans_times_force_pycuda(rp, fp, eta, a, mode=mode)
        ts = []
        for _ in range(20):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mb.single_wall_mobility_trans_times_force_pycuda(rp, fp, eta, a, mode=mode)
            ts.append(time.perf_counter() - t0)
        out["e2e_" + mode] = {"ms": float(np.median(ts)) * 1e3, "gpairs": n * n / float(np.median(ts)) / 1e9}
    threads = os.cpu_count() or 1
    wall.uf_symmetric_fast(r, f, eta, a, threads=threads)
    ts = []
    t_end = time.perf_counter() + cpu_seconds
    while len(ts) < 5 or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        wall.uf_symmetric_fast(r, f, eta, a, threads=threads)
        ts.append(time.perf_counter() - t0)
    med = float(np.median(ts))
    out["cpu_port"] = {"ms": med * 1e3, "gpairs": n * n / med / 1e9, "cores": threads, "products_timed": len(ts)}
    for mode in ("fp64", "df64"):
        out["speedup_e2e_%s_vs_cpu_port" % mode] = out["cpu_port"]["ms"] / out["e2e_" + mode]["ms"]
    return out


def solve_breakdown(fn):
    """Run fn() (one solve) with tracing on and split its device time by class: whole solve (first to last
    launch, host gaps included), preconditioner build, device-resident GMRES restart cycles (one graph
    launch each: operator applications and fused Arnoldi steps), or, host-driven, the operator applications
    (A P^-1 as graph replays) and Krylov vector work; refinement residuals; the rest is small kernels and
    host round trips."""
    from rigidmultiblobswall_gb300 import _native
    names = {1: "krylov_vector_ms", 3: "operator_ms", 4: "refine_residual_ms", 5: "pc_build_ms", 6: "solve_ms",
             7: "device_cycle_ms"}
    _native.trace_enable(True)
    for k in range(8):
        _native.trace_read(k, reset=True)
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = fn()
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1e3
    out = {"wall_ms": wall_ms}
    for k, nm in names.items():
        ms, cnt = _native.trace_read(k, reset=True)
        out[nm] = ms
        out[nm.replace("_ms", "_count")] = cnt
    for k in (0, 2):
        _native.trace_read(k, reset=True)
    _native.trace_bytes(1, reset=True)
    _native.trace_enable(False)
    out["other_in_solve_ms"] = out["solve_ms"] - out["operator_ms"] - out["krylov_vector_ms"] - \
        out["refine_residual_ms"] - out["device_cycle_ms"]
    out["outside_solve_ms"] = wall_ms - out["solve_ms"] - out["pc_build_ms"]
    return res, out


def train_nearfield(shell, a, z_range, dev, n_clusters=1024, steps=2000, seed=11):
    """Message-passing near-field network for one shell type: clusters of 2..8 bodies (centre distances
    2R+2a .. NF_CUTOFF_R, heights in z_range) whose pair couplings the plain method computes on the GPU, then Adam
    on the GPU.  Returns (model, info)."""
    import torch
    from rigidmultiblobswall_gb300 import nearfield as nf
    R = float(np.linalg.norm(shell[0]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    graphs = nf.cluster_training_data(shell, a, 1.0, n_clusters, d_range=(2 * R + 2 * a, NF_CUTOFF_R * R), z_range=z_range,
                                      seed=seed, device=dev)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    model = nf.NearfieldModel(body_radius=R, cutoff=NF_CUTOFF_R * R, seed=2)
    hist = model.train(graphs, steps=steps, lr=2e-3)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return model, {"clusters": n_clusters, "bodies_per_cluster": [2, 8], "graphs": len(graphs),
                   "pairs": int(sum(g.n_band for g in graphs)), "data_ms": (t1 - t0) * 1e3,
                   "train_ms": (t2 - t1) * 1e3, "steps": steps, "loss_first": float(hist[:10].mean()),
                   "loss_last": float(hist[-50:].mean())}


def solver_metrics(dev, reps=2):
    """Secondary: the 256-shell mobility solve (GMRES + block-diagonal PC to a
    1e-8 relative residual) in FP64 and mixed precision, and one Brownian
    Euler-Maruyama step of 1024 12-blob shells (Lanczos 1e-3 + GMRES 1e-8)."""
    import torch
    from rigidmultiblobswall_gb300 import integrator
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    out = {}
    s2 = S.shells_42_256()
    sys2 = RigidSystem([42] * s2.n_bodies, s2.eta, s2.a, device=dev)
    sys2.set_configuration(s2.r_vectors(), s2.locations)
    FT = np.zeros((s2.n_bodies, 6))
    FT[:, 2] = -1.0
    sols = {}
    for mode in ("fp64", "mixed"):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sys2.build_pc(mode=mode)
            sol, info, its, rr = integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode=mode)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        sols[mode] = sol.cpu().numpy()
        out["solve_shells42x256_%s" % mode] = {"ms": best * 1e3, "iterations": its, "relres_fp64": rr, "info": info}
    # the same mixed solve with the per-iteration operator launched kernel by kernel instead of as a
    # captured CUDA graph
    from rigidmultiblobswall_gb300 import _native
    _native.use_graphs(False)
    best = None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sys2.build_pc(mode="mixed")
        _, _, its_ng, _ = integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode="mixed")
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    _native.use_graphs(True)
    out["solve_shells42x256_mixed_without_graphs"] = {"ms": best * 1e3, "iterations": its_ng}
    # near-field augmented preconditioner: exact pairs below NF_EXACT_R body radii, learned beyond
    from rigidmultiblobswall_gb300 import nearfield as nf
    R2 = float(np.linalg.norm(s2.shell[0]))
    model42, out["nearfield_training_shells42"] = train_nearfield(s2.shell, s2.a, (1.1 * R2, 5 * R2), dev)
    for mode in ("fp64", "mixed"):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sys2.build_pc(mode=mode)
            pairs = model42.attach(sys2, exact_cutoff=NF_EXACT_R * R2)
            sol, info, its, rr = integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode=mode)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        nf.detach(sys2)
        sols[mode + "_nf"] = sol.cpu().numpy()
        out["solve_shells42x256_%s_nearfield" % mode] = {"ms": best * 1e3, "iterations": its, "relres_fp64": rr,
                                                          "info": info, "pairs_exact_learned": list(pairs)}
    # where the mixed solve's time goes (PC build + solve, traced by class)
    def _mixed():
        sys2.build_pc(mode="mixed")
        return integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode="mixed")
    _mixed()
    _, out["solve_shells42x256_mixed_breakdown"] = solve_breakdown(_mixed)
    # the preconditioner apply (256 126 x 126 blocks: 16-33 MB, L2-resident)
    out["pc_apply_shells42x256"] = pc_apply_roofline(sys2)
    # bandwidth of the Arnoldi vector work (33,792-long vectors: the basis stays in L2)
    sys2.build_pc()
    _, out["solve_shells42x256_mixed_arnoldi"] = arnoldi_traffic(
        lambda: integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode="mixed"))
    # errors judged by the oracle: its FP64 residual |b - A x| / |b| of every returned solution (all-pairs
    # product of oracle/wall_oracle.c, K and the operator of oracle/rigid.py) and the body velocities of
    # its own solve (restarted right-preconditioned GMRES with the block-diagonal preconditioner)
    from oracle import rigid as orc
    n3 = 3 * sys2.n_blobs
    orig = orc.Rigid(s2.r_vectors(), s2.locations, sys2.offsets, s2.eta, s2.a)
    rhs = np.concatenate([np.zeros(n3), -FT.reshape(-1)])
    nrm = np.linalg.norm(rhs)
    xo, ito, _ = orc.gmres_right(orig.apply, orig.apply_pc, rhs / nrm, tol=1e-8)
    uo = (xo * nrm)[n3:]
    u64 = sols["fp64"][n3:]
    for key, sk in (("fp64", "solve_shells42x256_fp64"), ("mixed", "solve_shells42x256_mixed"),
                    ("fp64_nf", "solve_shells42x256_fp64_nearfield"),
                    ("mixed_nf", "solve_shells42x256_mixed_nearfield")):
        x = sols[key]
        out[sk]["relres_oracle"] = float(np.linalg.norm(rhs - orig.apply(x)) / nrm)
        out[sk]["velocity_rel_err_vs_oracle"] = float(np.linalg.norm(x[n3:] - uo) / np.linalg.norm(uo))
        if key != "fp64":
            out[sk]["velocity_rel_err_vs_fp64"] = float(np.linalg.norm(x[n3:] - u64) / np.linalg.norm(u64))
    out["solve_shells42x256_oracle_iterations"] = ito
    out["solve_shells42x256_speedup_mixed"] = out["solve_shells42x256_fp64"]["ms"] / \
        out["solve_shells42x256_mixed"]["ms"]
    out["solve_shells42x256_speedup_mixed_nearfield"] = out["solve_shells42x256_fp64"]["ms"] / \
        out["solve_shells42x256_mixed_nearfield"]["ms"]
    # Brownian step, 1024 shells x 12 blobs
    s3 = S.shells_12_1024()
    sys3 = RigidSystem([12] * s3.n_bodies, s3.eta, s3.a, device=dev)
    FT3 = np.zeros((s3.n_bodies, 6))
    FT3[:, 2] = -1.0
    z = torch.randn(3 * s3.n_blobs, generator=torch.Generator(device=dev).manual_seed(3), dtype=torch.float64,
                    device=dev)
    vel = {}
    R3 = float(np.linalg.norm(s3.shell[0]))
    model12, out["nearfield_training_shells12"] = train_nearfield(s3.shell, s3.a, (1.1 * R3, 5 * R3), dev)
    # mixed_nearfield: exact couplings below NF_EXACT_R, learned ones from there to NF_CUTOFF_R;
    # mixed_exact: the exact part alone; mixed_learned: learned couplings for every pair below NF_CUTOFF_R
    # (no exact part); mixed_exact_all: exact couplings for every pair below NF_CUTOFF_R (no network)
    arms3 = {"fp64": None, "mixed": None, "mixed_nearfield": (model12, NF_EXACT_R * R3),
             "mixed_exact": (None, NF_EXACT_R * R3), "mixed_learned": (model12, 0.0),
             "mixed_exact_all": (None, NF_ALL_EXACT_R * R3)}
    for mode, nfa in arms3.items():
        best = None
        for _ in range(reps):
            st = integrator.BrownianStepper(sys3, s3.locations, s3.quaternions,
                                            np.tile(s3.shell, (s3.n_bodies, 1)), kT=1.0,
                                            mode=mode.split("_")[0], nearfield=nfa)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = st.step(1e-3, FT3, z=z)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        vel[mode] = res["velocities"].cpu().numpy()
        out["bd_step_shells12x1024_%s" % mode] = {"ms": best * 1e3, "lanczos_iterations": res["lanczos_iterations"],
                                                  "gmres_iterations": res["gmres_iterations"],
                                                  "relres_fp64": res["relres"]}
    for mode in ("mixed", "mixed_nearfield", "mixed_exact", "mixed_learned", "mixed_exact_all"):
        out["bd_step_shells12x1024_" + mode]["velocity_rel_err_vs_fp64"] = float(
            np.linalg.norm(vel[mode] - vel["fp64"]) / np.linalg.norm(vel["fp64"]))
    out["bd_step_ms_learned_vs_blockdiag"] = {
        "block_diag_fp64": out["bd_step_shells12x1024_fp64"]["ms"],
        "block_diag_mixed": out["bd_step_shells12x1024_mixed"]["ms"],
        "learned_mixed": out["bd_step_shells12x1024_mixed_nearfield"]["ms"],
        "exact_only_mixed": out["bd_step_shells12x1024_mixed_exact"]["ms"],
        "learned_only_mixed": out["bd_step_shells12x1024_mixed_learned"]["ms"],
        "exact_all_mixed": out["bd_step_shells12x1024_mixed_exact_all"]["ms"]}
    # every time integrator, one step of 1024 shells x 12 blobs (mixed precision,
    # GMRES and Lanczos tolerance 1e-8, force (0,0,-1) per body, kT = 1, dt = 1e-3)
    FT3t = torch.as_tensor(FT3, device=dev).reshape(-1, 3)
    sch = {}
    for scheme in integrator.QuaternionIntegrator.SCHEMES:
        qi = integrator.QuaternionIntegrator(sys3, scheme, s3.locations, s3.quaternions,
                                             np.tile(s3.shell, (s3.n_bodies, 1)), tolerance=1e-8, kT=1.0,
                                             mode="mixed", seed=5)
        qi.force_torque_calculator = lambda s, r: FT3t
        qi.advance_time_step(1e-3, step=0)  # warm-up (and the second step of the two-step schemes)
        d0, s0 = qi.det_iterations_count, qi.stoch_iterations_count
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        qi.advance_time_step(1e-3, step=1)
        torch.cuda.synchronize()
        sch[scheme] = {"ms": (time.perf_counter() - t0) * 1e3, "gmres_iterations": qi.det_iterations_count - d0,
                       "lanczos_iterations": qi.stoch_iterations_count - s0}
        qi.close()
    out["schemes_shells12x1024_mixed_step"] = sch
    return out


def cpu_solve_baselines():
    """The reference's solve path on the host cores: its Python structure (restated by the oracle:
    linear_operator_rigid, the block-diagonal preconditioner, right-preconditioned restarted GMRES,
    Lanczos; multi_bodies.py:424-471, 752-903, general_application_utils.py:514-635,
    stochastic_forcing.py:112-264) with the oracle's restatement of the reference C++ product
    (mobility/mobility.cpp:256-430, symmetric loop, OpenMP over all host cores) as the matvec - the
    configuration a user of the reference runs with mobility_vector_prod_implementation = C++.
    256-shell solve to 1e-8, and one 1024 x 12-blob Euler-Maruyama step (Lanczos 1e-3, GMRES 1e-8)."""
    from oracle import rigid as orc
    from oracle import wall
    from rigidmultiblobswall_gb300 import suspensions as S
    threads = os.cpu_count() or 1

    class FastRigid(orc.Rigid):
        def mobility(self, v):
            return wall.uf_symmetric_fast(self.r, v, self.eta, self.a, threads=threads)

    out = {}
    s2 = S.shells_42_256()
    r2 = s2.r_vectors()
    o = FastRigid(r2, s2.locations, 42 * np.arange(s2.n_bodies + 1), s2.eta, s2.a)
    FT = np.zeros((s2.n_bodies, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * len(r2)), -FT.reshape(-1)])
    t0 = time.perf_counter()
    o.build_pc()
    x, it, rel = orc.gmres_right(o.apply, o.apply_pc, rhs / np.linalg.norm(rhs), tol=1e-8)
    dt = time.perf_counter() - t0
    out["solve_shells42x256"] = {"ms": dt * 1e3, "iterations": it, "relres": rel, "cores": threads,
                                 "kind": "port"}
    s3 = S.shells_12_1024()
    r3 = s3.r_vectors()
    o3 = FastRigid(r3, s3.locations, 12 * np.arange(s3.n_bodies + 1), s3.eta, s3.a)
    FT3 = np.zeros((s3.n_bodies, 6))
    FT3[:, 2] = -1.0
    z = np.random.default_rng(3).standard_normal(3 * len(r3))
    dtm = 1e-3
    t0 = time.perf_counter()
    o3.build_pc()
    raw, itl = orc.lanczos(o3.mobility_pc, z, factor=np.sqrt(2.0 / dtm), tol=1e-3)
    noise = o3.P_inv_mult(raw)
    b3 = np.concatenate([-noise, -FT3.reshape(-1)])
    nrm = np.linalg.norm(b3)
    x3, it3, rel3 = orc.gmres_right(o3.apply, o3.apply_pc, b3 / nrm, tol=1e-8)
    orc.em_update(s3.locations, s3.quaternions, (x3 * nrm)[3 * len(r3):], dtm)
    dt3 = time.perf_counter() - t0
    out["bd_step_shells12x1024"] = {"ms": dt3 * 1e3, "lanczos_iterations": itl, "gmres_iterations": it3,
                                    "relres": rel3, "cores": threads, "kind": "port"}
    out["sample"] = ("one full solve / step each; oracle numpy restatement of the reference's Python solve path "
                     "with the oracle's restatement of the reference C++ symmetric product as the matvec")
    return out


def oracle_residual_sampled(r, locs, offsets, eta, a, sol, FT, n_rows=1024, seed=0):
    """The oracle's relative residual |b - A x| / |b| of a rigid solution, estimated from every body row
    (-K^T lambda = -F) and n_rows sampled blob rows (M lambda - K U = 0, the oracle's all-source product on
    those rows); the sampled part is scaled up to all blob rows."""
    from oracle import wall
    from oracle import rigid as orc
    N = len(r)
    lam, U = sol[:3 * N], sol[3 * N:]
    Ks = orc.K_bodies(r, locs, offsets)
    rb = orc.KT_mult(Ks, offsets, lam) - FT.reshape(-1)
    rows = np.sort(np.random.default_rng(seed).choice(N, min(n_rows, N), replace=False))
    Ml = wall.wall_product("uf", r, lam, eta, a, rows=rows)
    body = np.searchsorted(offsets, rows, side="right") - 1
    d = r[rows] - locs[body]
    KU = U.reshape(-1, 6)[body, :3] + np.cross(U.reshape(-1, 6)[body, 3:], d)
    rs = Ml - KU.reshape(-1)
    est = np.sqrt(rb @ rb + (N / rows.size) * (rs @ rs))
    return float(est / np.linalg.norm(FT)), int(rows.size)


def cfg5_metrics(dev, modes=("fp64", "mixed", "mixed+exact", "mixed+learned", "mixed+learned_band",
                             "mixed+exact+learned", "mixed+exact_all")):
    """4096 42-blob shells at area fraction 0.3, force (0,0,-1) per body: preconditioned GMRES to a 1e-8
    relative residual, on one GPU.  Arms: plain block-diagonal FP64 (the baseline), mixed precision, and
    mixed precision with the near-field augmented preconditioner - exact blob-level couplings below
    NF_EXACT_R only ("exact"), learned mode couplings of every pair below NF_CUTOFF_R ("learned"), of the
    outer band NF_EXACT_R..NF_CUTOFF_R only ("learned_band"), exact below NF_EXACT_R with learned from there
    to NF_CUTOFF_R ("exact+learned"), and exact couplings of every pair below NF_CUTOFF_R without the
    network ("exact_all").
    Each arm's time covers its preconditioner build (FP64 or FP32), the near-field
    attach and the solve; the network is trained once before (time reported).  Every solution's relative
    residual is also estimated by the oracle (all body rows, 1024 sampled blob rows)."""
    import torch
    from rigidmultiblobswall_gb300 import integrator
    from rigidmultiblobswall_gb300 import nearfield as nf
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    s5 = S.shells_42_4096()
    r5 = s5.r_vectors()
    sys5 = RigidSystem([42] * s5.n_bodies, s5.eta, s5.a, device=dev)
    sys5.set_configuration(r5, s5.locations)
    FT = np.zeros((s5.n_bodies, 6))
    FT[:, 2] = -1.0
    R5 = float(np.linalg.norm(s5.shell[0]))
    out = {"workload": "4096 shells x 42 blobs = 172,032 blobs, area fraction 0.3, z in [1.1R, 3R], F=(0,0,-1)",
           "tol": 1e-8, "restart": 60, "exact_cutoff": "%gR" % NF_EXACT_R,
           "learned_band": "%gR..%gR" % (NF_EXACT_R, NF_CUTOFF_R),
           "message_cutoff": "3R"}
    model = None
    if any("learned" in m for m in modes):
        model, out["nearfield_training"] = train_nearfield(s5.shell, s5.a, (1.1 * R5, 3 * R5), dev)
    sols = {}
    for mode in modes:
        parts = mode.split("+")
        base = parts[0]
        exact = "exact" in parts
        exact_all = "exact_all" in parts
        band_only = "learned_band" in parts
        learned = band_only or "learned" in parts
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sys5.build_pc(mode="mixed" if base == "mixed" else base)
        pairs = None
        if learned:
            pairs = model.attach(sys5, exact_cutoff=NF_EXACT_R * R5 if exact else 0.0,
                                 learned_from=NF_EXACT_R * R5 if band_only else 0.0)
        elif exact or exact_all:
            pairs = nf.attach_exact(sys5, (NF_ALL_EXACT_R if exact_all else NF_EXACT_R) * R5)
        sol, info, its, rr = integrator.solve_mobility_problem(sys5, FT, tol=1e-8, mode=base)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if pairs is not None:
            nf.detach(sys5)
        x = sol.cpu().numpy()
        sols[mode] = x[3 * sys5.n_blobs:]
        est, nrows = oracle_residual_sampled(r5, s5.locations, sys5.offsets, s5.eta, s5.a, x, FT)
        out[mode] = {"ms": dt * 1e3, "iterations": its, "relres": rr, "info": info,
                     "oracle_relres_estimate": est, "oracle_rows_sampled": nrows}
        if pairs is not None:
            out[mode]["pairs_exact_learned"] = list(pairs)
    ref = sols.get("fp64")
    for mode, u in sols.items():
        if ref is not None:
            out[mode]["velocity_rel_err_vs_fp64"] = float(np.linalg.norm(u - ref) / np.linalg.norm(ref))
    # the preconditioner apply at this size: 4096 blocks of 126 x 126 (0.26 GB in FP32, 0.52 GB in FP64
    # per apply, beyond the L2)
    nf.detach(sys5)
    sys5.build_pc(mode="mixed")
    out["pc_apply"] = pc_apply_roofline(sys5, reps=10)
    if "fp64" in out:
        for mode in modes:
            if mode != "fp64":
                out["speedup_%s_vs_fp64" % mode] = out["fp64"]["ms"] / out[mode]["ms"]
    for m1, m2 in (("mixed+exact+learned", "mixed+exact"), ("mixed+learned", "mixed"),
                   ("mixed+learned_band", "mixed"), ("mixed+exact+learned", "mixed+exact_all")):
        if m1 in out and m2 in out:
            out["gain_%s_over_%s" % (m1, m2)] = {"ms_ratio": out[m2]["ms"] / out[m1]["ms"],
                                                 "iterations": [out[m2]["iterations"], out[m1]["iterations"]]}
    sys5.close()
    return out


def large_solve(args):
    """--large: only the 4096-shell solve comparison (modes from --large-modes), as one JSON line."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    clocks = ClockSampler(0)
    clocks.start()
    out = cfg5_metrics(dev, tuple(args.large_modes.split(",")))
    out["clocks"] = clocks.stop()
    print(json.dumps(out))


def batched_metrics(dev, nrhs=16):
    """64 independent suspensions of 42-blob shells (16..512 bodies each, seeded):
    stochastic block-diagonal preconditioner, 16 Lanczos right-hand sides per
    suspension (tolerance 1e-3, mixed precision, lockstep over all
    (suspension, RHS) pairs) and every suspension's mobility solve to 1e-8
    (lockstep batched GMRES, mixed precision with df64 refinement)."""
    import torch
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    susps = S.shells_42_batch()
    counts = [s.n_bodies for s in susps]
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    sysb = RigidSystem([42] * sum(counts), susps[0].eta, susps[0].a, device=dev)
    sysb.set_configuration(r, locs)
    sysb.set_suspensions(counts)
    pairs = int(sum((42 * c) ** 2 for c in counts))
    out = {"workload": "64 suspensions, 16..512 42-blob shells each (%d bodies, %d blobs, %.3g pairs/product)"
           % (sum(counts), sysb.n_blobs, pairs)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sysb.build_pc(stochastic=True, mode="mixed")
    torch.cuda.synchronize()
    out["pc_build_ms"] = (time.perf_counter() - t0) * 1e3
    Z = torch.randn(nrhs, 3 * sysb.n_blobs, generator=torch.Generator(device=dev).manual_seed(4),
                    dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    noise, itl = sysb.lanczos_batched(Z, factor=np.sqrt(2.0 / 1e-3), tol=1e-3, mode="mixed")
    torch.cuda.synchronize()
    out["lanczos_16rhs_ms"] = (time.perf_counter() - t0) * 1e3
    out["lanczos_iterations_min_max"] = [int(itl.min()), int(itl.max())]
    FT = np.zeros((sum(counts), 6))
    FT[:, 2] = -1.0
    rhs = torch.cat([torch.zeros(3 * sysb.n_blobs, dtype=torch.float64, device=dev),
                     -torch.tensor(FT.reshape(-1), device=dev)])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, its, rr, stt = sysb.solve_batched(rhs, tol=1e-8, mode="mixed")
    torch.cuda.synchronize()
    out["solve_ms"] = (time.perf_counter() - t0) * 1e3
    out["solve_iterations_min_max"] = [int(its.min()), int(its.max())]
    out["solve_relres_max"] = float(rr.max())
    out["all_converged"] = bool((stt == 0).all())
    # the same solve again, traced: bandwidth of the segmented Arnoldi work (2.1 M-long vectors, basis > L2)
    _, out["solve_arnoldi"] = arnoldi_traffic(lambda: sysb.solve_batched(rhs, tol=1e-8, mode="mixed"))
    # roofline of the 16-RHS Lanczos: the multi-right-hand-side pair kernel's share of the time and its
    # FP32 issue rate (launched kernel by kernel, traced).  Pair-RHS evaluations: the kernel runs a pass
    # of 16 right-hand sides of a suspension while any of them still iterates (it + 1 operator
    # applications for it iterations), over n_k^2 blob pairs.
    from rigidmultiblobswall_gb300 import _native
    _native.use_graphs(False)
    _native.trace_enable(True)
    _native.trace_read(0, reset=True)
    _native.trace_read(1, reset=True)
    _native.trace_bytes(1, reset=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, itl2 = sysb.lanczos_batched(Z, factor=np.sqrt(2.0 / 1e-3), tol=1e-3, mode="mixed")
    torch.cuda.synchronize()
    lz_ms = (time.perf_counter() - t0) * 1e3
    pair_ms, pair_launches = _native.trace_read(0, reset=True)
    step_ms, step_launches = _native.trace_read(1, reset=True)
    _native.trace_bytes(1, reset=True)
    for k in (2, 3, 4, 5, 6, 7):
        _native.trace_read(k, reset=True)
    _native.trace_enable(False)
    _native.use_graphs(True)
    hbm, hsrc = hbm_peak_gbs()
    it = np.asarray(itl2).reshape(nrhs, len(counts))
    nblob = 42 * np.asarray(counts, dtype=np.float64)
    prhs = 0.0
    for p in range(0, nrhs, 16):
        w = min(16, nrhs - p)
        prhs += float(((it[p:p + w].max(axis=0) + 1) * nblob ** 2).sum()) * (16 if w > 8 else 8)
    # algorithmic traffic of the Lanczos steps: a segment (right-hand side q of suspension k, 3 n_k long)
    # that reports it iterations ran steps i = 0..it, step i moving (2i + 4) x 3 n_k doubles (full
    # reorthogonalisation over V_0..V_i)
    step_bytes = float((24.0 * nblob[None, :] * (it + 1) * (it + 4)).sum())
    peak32 = _native.fma_peak(False)
    ipr = MULTI16_INST_PER_PAIR_RHS
    out["lanczos_16rhs_roofline"] = {
        "lanczos_ms_without_graphs": lz_ms, "pair_kernel_ms": pair_ms, "pair_kernel_launches": pair_launches,
        "pair_kernel_share": pair_ms / lz_ms, "pair_rhs_evaluated": prhs,
        "tpair_rhs_per_s": prhs / (pair_ms * 1e-3) / 1e12,
        "issued_inst_per_pair_rhs": ipr, "fp32_issue_frac": prhs * ipr / (pair_ms * 1e-3) / (peak32 / 2.0),
        "note": "issued instructions per pair-RHS from the ncu capture of wall_pair_multi_kernel (16 RHS)",
        "lanczos_step_kernel": {"launches": step_launches, "ms": step_ms, "gbytes": step_bytes / 1e9,
                                "gbs": step_bytes / (step_ms * 1e-3) / 1e9 if step_ms > 0 else None,
                                "frac_of_hbm": step_bytes / (step_ms * 1e-3) / 1e9 / hbm if step_ms > 0 else None,
                                "hbm_peak_gbs": hbm, "peak_source": hsrc,
                                "bytes_per_step": "(2i + 4) x 3N doubles (full reorthogonalisation over V_0..V_i)"}}
    return out


def single_product(args):
    """One wall product on the 256-shell workload (the default split of the autotuner's cache, i.e. the
    symmetric kernel at this size, for every block and precision mode): CUDA-event time per step, L2 flushed between
    steps."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    from rigidmultiblobswall_gb300 import mobility as mb
    B.build()
    kind, mode = args.product.split(":")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s, r, f = workload()
    rt = torch.tensor(r, device=dev)
    ft = torch.tensor(f, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup - 2, 0)):
        mb.wall_product(kind, rt, ft, s.eta, s.a, mode=mode)
    res = time_product(kind, mode, rt, ft, None, s.eta, s.a, args.steps, flush, torch.cuda.current_stream(dev))
    print(json.dumps({"metric": "M_%s product Gpairs/s" % kind.upper(), "mode": mode,
                      "workload": "256 shells x 42 blobs = 10,752 blobs, forces N(0,1), seed 1",
                      "n_blobs": len(r), "steps": args.steps, **res}))


def multi_product(args):
    """The multi-right-hand-side M_UF product (mixed precision) on N random blobs above the wall
    (suspensions.blobs_wall_matvec, seed 3) with NRHS N(0,1) vectors: CUDA-event time per product after
    --warmup products (inputs of NRHS x 3N doubles; pair work far above L2 traffic)."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    from rigidmultiblobswall_gb300 import mobility as mb
    from rigidmultiblobswall_gb300 import suspensions as S
    B.build()
    n, nrhs = (int(x) for x in args.multi.split(":"))
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    r, _, eta, a = S.blobs_wall_matvec(n, seed=3)
    rt = torch.tensor(r, device=dev)
    V = torch.randn(nrhs, 3 * n, generator=torch.Generator(device=dev).manual_seed(5), dtype=torch.float64,
                    device=dev)
    for _ in range(args.warmup):
        mb.uf_multi(rt, V, eta, a)
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        mb.uf_multi(rt, V, eta, a)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    print(json.dumps({"metric": "multi-RHS M_UF product T pair-RHS/s", "mode": "mixed", "n_blobs": n,
                      "nrhs": nrhs, "steps": args.steps, "ms": ms,
                      "tpair_rhs_per_s": n * n * nrhs / (ms * 1e-3) / 1e12}))


def krylov_probe():
    """The 4096-shell mixed solve with every fused Arnoldi step launched and traced on its own (graphs off)
    and the product scratch capped at 1 GiB (one-sided pair kernels, small device footprint): one JSON line
    with the solve time and the Arnoldi steps' time, algorithmic bytes and bandwidth."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    from rigidmultiblobswall_gb300 import _native, integrator
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.set_scratch_limit(1 << 30)
    s5 = S.shells_42_4096()
    sys5 = RigidSystem([42] * s5.n_bodies, s5.eta, s5.a, device=dev)
    sys5.set_configuration(s5.r_vectors(), s5.locations)
    FT = np.zeros((s5.n_bodies, 6))
    FT[:, 2] = -1.0
    sys5.build_pc(mode="mixed")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    (sol, info, its, rr), arn = arnoldi_traffic(
        lambda: integrator.solve_mobility_problem(sys5, FT, tol=1e-8, mode="mixed"))
    torch.cuda.synchronize()
    print(json.dumps({"solve_ms": (time.perf_counter() - t0) * 1e3, "iterations": its, "relres": rr,
                      "arnoldi": arn}))


def lanczos_probe(nsusp=64):
    """The 16-right-hand-side Lanczos of the first nsusp of the 64 uneven suspensions (mixed precision,
    tolerance 1e-3) with graphs off, so that every fused Lanczos step is a launch of its own: one JSON line
    with the run's time and the step kernel's traced time, algorithmic bytes and bandwidth."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    from rigidmultiblobswall_gb300 import _native
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    susps = S.shells_42_batch()[:max(1, nsusp)]
    counts = [s.n_bodies for s in susps]
    sysb = RigidSystem([42] * sum(counts), susps[0].eta, susps[0].a, device=dev)
    sysb.set_configuration(np.concatenate([s.r_vectors() for s in susps]),
                           np.concatenate([s.locations for s in susps]))
    sysb.set_suspensions(counts)
    sysb.build_pc(stochastic=True, mode="mixed")
    nrhs = 16
    Z = torch.randn(nrhs, 3 * sysb.n_blobs, generator=torch.Generator(device=dev).manual_seed(4),
                    dtype=torch.float64, device=dev)
    _native.use_graphs(False)
    _native.trace_enable(True)
    _native.trace_read(1, reset=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, itl = sysb.lanczos_batched(Z, factor=np.sqrt(2.0 / 1e-3), tol=1e-3, mode="mixed")
    torch.cuda.synchronize()
    lz_ms = (time.perf_counter() - t0) * 1e3
    step_ms, step_launches = _native.trace_read(1, reset=True)
    for k in range(8):
        _native.trace_read(k, reset=True)
    _native.trace_bytes(1, reset=True)
    _native.trace_enable(False)
    _native.use_graphs(True)
    it = np.asarray(itl).reshape(nrhs, len(counts))
    nblob = 42 * np.asarray(counts, dtype=np.float64)
    step_bytes = float((24.0 * nblob[None, :] * (it + 1) * (it + 4)).sum())
    print(json.dumps({"suspensions": len(counts), "blobs": int(sysb.n_blobs), "lanczos_ms": lz_ms,
                      "iterations_min_max": [int(it.min()), int(it.max())],
                      "step_launches": step_launches, "step_ms": step_ms, "step_gbytes": step_bytes / 1e9,
                      "step_gbs": step_bytes / (step_ms * 1e-3) / 1e9 if step_ms > 0 else None}))


def bd_probe():
    """One Brownian step of the 1024 12-blob shells (mixed precision, Lanczos 1e-3, GMRES 1e-8), plain and
    with the near field (exact below NF_EXACT_R, learned to NF_CUTOFF_R): a warm-up step, a timed step, then
    one step with graphs off (every kernel a launch of its own) inside the NVTX range "bd_step_<arm>", which
    ncu --nvtx --nvtx-include "bd_step_<arm>/" lists launch by launch.  One JSON line with the times."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    from rigidmultiblobswall_gb300 import integrator
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s3 = S.shells_12_1024()
    sys3 = RigidSystem([12] * s3.n_bodies, s3.eta, s3.a, device=dev)
    FT3 = np.zeros((s3.n_bodies, 6))
    FT3[:, 2] = -1.0
    z = torch.randn(3 * s3.n_blobs, generator=torch.Generator(device=dev).manual_seed(3), dtype=torch.float64,
                    device=dev)
    R3 = float(np.linalg.norm(s3.shell[0]))
    model12, _ = train_nearfield(s3.shell, s3.a, (1.1 * R3, 5 * R3), dev)
    from rigidmultiblobswall_gb300 import _native
    out = {}

    def step(nfa):
        st = integrator.BrownianStepper(sys3, s3.locations, s3.quaternions, np.tile(s3.shell, (s3.n_bodies, 1)),
                                        kT=1.0, mode="mixed", nearfield=nfa)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = st.step(1e-3, FT3, z=z)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, res

    for name, nfa in (("mixed", None), ("mixed_nearfield", (model12, NF_EXACT_R * R3))):
        step(nfa)
        ms, res = step(nfa)
        _native.use_graphs(False)
        torch.cuda.nvtx.range_push("bd_step_" + name)
        ms_ng, _ = step(nfa)
        torch.cuda.nvtx.range_pop()
        _native.use_graphs(True)
        out[name] = {"ms": ms, "ms_without_graphs": ms_ng, "gmres_iterations": res["gmres_iterations"],
                     "lanczos_iterations": res["lanczos_iterations"]}
    print(json.dumps(out))


def pc_probe():
    """The block-diagonal preconditioner of the 4096-shell suspension (FP32 build, the mixed solves'):
    the FP64 and FP32 applies timed over repeated calls, one JSON line (pc_apply_roofline)."""
    import torch
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    from rigidmultiblobswall_gb300 import suspensions as S
    from rigidmultiblobswall_gb300.rigid import RigidSystem
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s5 = S.shells_42_4096()
    sys5 = RigidSystem([42] * s5.n_bodies, s5.eta, s5.a, device=dev)
    sys5.set_configuration(s5.r_vectors(), s5.locations)
    sys5.build_pc(mode="mixed")
    print(json.dumps({"workload": "4096 shells x 42 blobs, 4096 126 x 126 blocks", **pc_apply_roofline(sys5, reps=20)}))


def main():
    args = parse()
    if args.krylov_probe:
        krylov_probe()
        return
    if args.pc_probe:
        pc_probe()
        return
    if args.bd_probe:
        bd_probe()
        return
    if args.lanczos_probe is not None:
        lanczos_probe(args.lanczos_probe)
        return
    if args.large:
        large_solve(args)
        return
    if args.product:
        single_product(args)
        return
    if args.multi:
        multi_product(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist
    from rigidmultiblobswall_gb300 import build as B
    B.build()
    from rigidmultiblobswall_gb300 import _native
    from rigidmultiblobswall_gb300 import mobility as mb
    ws, rank = dist_setup()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)

    s, r, f = workload()
    n = len(r)
    eta, a = s.eta, s.a
    rt = torch.tensor(r, device=dev)
    ft = torch.tensor(f, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    peak64 = _native.fma_peak(True)
    peak32 = _native.fma_peak(False)

    # ---- launch shape: the library's autotuner picks the pair grid's source split for this size
    tune = mb.autotune("uf", n, HEAD_MODE, reps=5)

    # ---- warm-up
    for _ in range(args.warmup):
        mb.wall_product("uf", rt, ft, eta, a, mode=HEAD_MODE)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()

    # ---- timed region: K steps of FP64 M.F with an L2 flush between steps
    clocks = ClockSampler(dev.index)
    clocks.start()
    _native.trace_enable(True)
    _native.trace_read(0, reset=True)
    evs = []
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = mb.wall_product("uf", rt, ft, eta, a, mode=HEAD_MODE)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    t_wall = time.perf_counter() - t_wall0
    step_ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    pair_ms_total, pair_launches = _native.trace_read(0, reset=True)
    _native.trace_enable(False)
    clk = clocks.stop()
    step_ms = reduce_step_ms(step_ms, ws, dev)
    ms_per_step = step_ms / args.steps
    value = aggregate_gpairs(step_ms, ws, args.steps, n)

    # ---- roofline of the dominant kernel (the df64 pair kernel; bound by the FP32/FMA pipe)
    pair_ms = pair_ms_total / max(pair_launches, 1)
    alg_tflops = n * n * FLOPS_PER_PAIR["uf"] / (pair_ms * 1e-3) / 1e12
    kernel = "symmetric" if tune["nchunks"] == -1 else "standard"
    ipp = DF64_UF_INST_PER_PAIR[kernel]
    peak_inst = peak32 / 2.0  # FMA-pipe thread instructions per second (one FFMA = 2 flops)
    roofline = {"bound": "fp32-pipe (issue)", "unit": "Tinst/s", "peak": peak_inst / 1e12,
                "achieved": (n * n * ipp / (pair_ms * 1e-3) / 1e12) if ipp else None,
                "frac": (n * n * ipp / (pair_ms * 1e-3) / peak_inst) if ipp else None,
                "traffic": DF64_UF_TRAFFIC_BYTES[kernel], "kernel": "wall_uf_df_sym_kernel" if kernel == "symmetric"
                else "wall_pair_df_kernel<UF>",
                "peak_source": "measured by rmw_fma_peak (FP32 FMA chains on all SMs) in this run, / 2 per FFMA",
                "pair_kernel_ms": pair_ms, "issued_inst_per_ordered_pair": ipp,
                "algorithmic_tflops_fp64_equivalent": alg_tflops, "flops_per_pair": FLOPS_PER_PAIR["uf"],
                "algorithmic_vs_measured_fp64_peak": alg_tflops / (peak64 / 1e12),
                # the reference's flops per pair (FP64 operations counted from its source) executed per
                # second, over the FP32 FMA peak of the pipe the df64 arithmetic runs on
                "algorithmic_frac_of_fp32_peak": alg_tflops / (peak32 / 1e12),
                "constants_source_sha256": DF64_UF_KERNEL_SOURCE_SHA}

    # ---- e2e through the public host-buffer API (copies inside the timed region)
    rp = torch.empty(r.shape, dtype=torch.float64).pin_memory().numpy()
    fp = torch.empty(f.shape, dtype=torch.float64).pin_memory().numpy()
    rp[:] = r
    fp[:] = f
    mb.single_wall_mobility_trans_times_force_pycuda(rp, fp, eta, a, mode=HEAD_MODE)
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u = mb.single_wall_mobility_trans_times_force_pycuda(rp, fp, eta, a, mode=HEAD_MODE)
        e2e_t.append(time.perf_counter() - t0)
    e2e = {"value": n * n / float(np.mean(e2e_t)) / 1e9, "unit": "Gpairs/s",
           "h2d_bytes_per_step": int(rp.nbytes + fp.nbytes), "d2h_bytes_per_step": int(u.nbytes)}

    # ---- secondary: every product in both precisions (same workload)
    products = {}
    for kind in (() if args.no_extras else ("uf", "ut", "wf", "wt")):
        for mode in ("fp64", "df64", "mixed"):
            mb.autotune(kind, n, mode, reps=3)
            res = time_product(kind, mode, rt, ft, None, eta, a, max(3, min(40, args.steps // 4)), flush, stream)
            peak = peak64 if mode in ("fp64", "df64") else peak32
            # algorithmic (reference) flops per second over the pipe peak of the mode's arithmetic
            # class; for df64 this is FP64-equivalent work over the FP64 peak (> 1 = faster than the
            # FP64 pipe could do it)
            res["alg_tflops"] = n * n * FLOPS_PER_PAIR[kind] / (res["pair_kernel_ms"] * 1e-3) / 1e12
            res["alg_frac_of_mode_peak"] = res["alg_tflops"] * 1e12 / peak
            products["%s_%s" % (kind, mode)] = {k: round(v, 6) for k, v in res.items()}

    # the force-and-torque product [U; W] = M [F; T] (in mixed one symmetric
    # fused pass over the pairs; in FP64 and df64 the sum of the four symmetric
    # single products) against the four single products called one by one
    if not args.no_extras:
        tt = torch.tensor(np.random.default_rng(7).standard_normal(3 * n), device=dev)
        for mode in ("fp64", "df64", "mixed"):
            reps = 3 if mode == "fp64" else 10

            def entry():
                return mb.wall_force_torque(rt, ft, tt, eta, a, mode=mode)

            def four():
                return [mb.wall_product(k, rt, v, eta, a, mode=mode) for k, v in (("uf", ft), ("ut", tt), ("wf", ft),
                                                                                 ("wt", tt))]
            res = {}
            for name, fn in (("force_torque_ms", entry), ("four_products_ms", four)):
                fn()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    fn()
                e1.record(stream)
                torch.cuda.synchronize()
                res[name] = e0.elapsed_time(e1) / reps
            res["gpairs"] = n * n / (res["force_torque_ms"] * 1e-3) / 1e9
            res["route"] = "symmetric fused kernel" if mode == "mixed" else "four symmetric products"
            products["force_torque_6n_%s" % mode] = {k: (round(v, 6) if isinstance(v, float) else v)
                                                      for k, v in res.items()}

    # source-target products with per-blob radii (the same blobs as sources and
    # targets, radii a (1 +- 20%)), and the single-radius free-surface product
    if not args.no_extras:
        rr = torch.tensor(a * np.random.default_rng(8).uniform(0.8, 1.2, n), device=dev)
        for geom in ("wall", "no_wall", "free_surface"):
            for mode in ("fp64", "df64", "mixed"):
                reps = 3 if mode == "fp64" else 10
                fn = lambda: mb.source_target_product(geom, rt, rt, ft, rr, rr, eta, mode=mode)  # noqa: E731
                fn()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                products["source_target_%s_%s" % (geom, mode)] = {"ms": round(ms, 6),
                                                                   "gpairs": round(n * n / (ms * 1e-3) / 1e9, 3)}
        for mode in ("fp64", "df64", "mixed"):
            fn = lambda: mb.free_surface_mobility_trans_times_force_gb300(rt, ft, eta, a, mode=mode)  # noqa: E731
            fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(5):
                fn()
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t0) * 1e3 / 5
            products["free_surface_%s" % mode] = {"ms": round(ms, 6), "gpairs": round(n * n / (ms * 1e-3) / 1e9, 3)}
        # the free-space (no wall) single-radius products (symmetric kernels at this size)
        for kind in ("uf", "wt"):
            for mode in ("fp64", "df64", "mixed"):
                reps = 3 if mode == "fp64" else 10
                fn = lambda: mb.no_wall_product(kind, rt, ft, eta, a, mode=mode)  # noqa: E731
                fn()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                products["no_wall_%s_%s" % (kind, mode)] = {"ms": round(ms, 6),
                                                            "gpairs": round(n * n / (ms * 1e-3) / 1e9, 3)}

    cfg1 = None if args.no_extras else cfg1_metrics(dev, flush, stream)
    solver = {} if args.no_extras else solver_metrics(dev)
    if not args.no_extras:
        solver["batched_64_suspensions"] = batched_metrics(dev)
        solver["cfg5_solve_shells42x4096"] = cfg5_metrics(dev)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(r, f, eta, a, args.cpu_seconds)
        if not args.no_extras:
            cb = cpu_solve_baselines()
            solver["cpu_baseline_solves"] = cb
            for key, gkey in (("solve_shells42x256", "solve_shells42x256_mixed"),
                              ("bd_step_shells12x1024", "bd_step_shells12x1024_mixed")):
                if gkey in solver:
                    solver[gkey]["cpu_baseline"] = cb[key]
                    solver[gkey]["speedup_vs_cpu_baseline"] = cb[key]["ms"] / solver[gkey]["ms"]

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "df64 (f64-accurate)", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD, "mode": HEAD_MODE, "n_blobs": n, "pairs_per_step": n * n, "eta": eta, "a": a,
                           "l2": "512 MB buffer written between timed steps (inputs 0.5 MB < L2)",
                           "launch_shape": {"kernel": kernel, "source_chunks": None if kernel == "symmetric"
                                            else tune["nchunks"], "chosen_by": "rmw_wall_autotune",
                                            "tuned_ms": tune["ms"],
                                            "standard_kernel_builtin_split_ms": tune["default_ms"]},
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": 3 * args.steps, "wall_s_timed_region": t_wall,
                "fp32_fma_peak_tflops": peak32 / 1e12, "fp64_fma_peak_tflops": peak64 / 1e12,
                "cfg1_plain_matvec_2048": cfg1, "products": products, "solver": solver}
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
