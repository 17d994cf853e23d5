"""Benchmark: query patches/s of the NNF hot path on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload large|medium|small|batch|stream] [--form learned|parallel|plain|openclopt]
                    [--iters N] [--no-compare] [--no-cpu-baseline]

A step is one full NNF of one image pair, from device-resident uint8 images to the device-resident
NNF. Forms: "plain" is the reference's method (PCA fit with the FP64 eigensolver, exact
projection, k-d tree, exact first row, row propagation, raw-patch re-rank); "parallel" is the BF16
form (subspace PCA with an FP64 Rayleigh-Ritz step, FP16 tensor-core projection, the same tree,
BF16 tensor-core natural-leaf tiles with exact FP32 re-rank, parallel propagation with exact
raw-patch verification); "learned" adds the trained offset-proposal network; "openclopt" is the
reference GPU backend's algorithm on this library's kernels. value = query patches
(A patch positions) per second over all ranks; distance_error = mean / p99 of d_found/d_exact - 1
over 4096 sampled pixels against the exact raw-patch nearest neighbour; "forms" times the other
forms on the same pair. e2e = the same through the public API from pinned host images to the host
NNF. The L2 cache (129 MB) is flushed between timed steps by writing 256 MB.

--impl reference times the CPU path (the oracle: a C restatement of the reference's OpenMP core with
OpenMP on all host cores, plus the numpy restatement of its PCA): every step is one complete fit
of the same pair by the reference's plain method (PCA fit, projection of both images, tree, the
whole row loop with the re-rank); nothing is extrapolated.

With --gpus 1 and no --no-compare, the line also carries "workloads": the 512x512 pair by the
plain method (patch 7, PCA 8, leaf 32, k 1), the 64 uneven pairs in one graph launch and the
1920x1080 frame stream, each with its own time and distance error.
"""
from __future__ import annotations

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

WORKLOADS = {
    # 2048x2048 flow-warped pair (seed 1): psize 9 (243-dim), PCA 16, leaf 64, k 4
    "large": dict(size=2048, seed=1, kind="flow", n_neighbors=4, psize=9, dim_reduced=16, leaf_size=64),
    # 512x512 affine pair (seed 0): psize 7 (147-dim), PCA 8, leaf 32, k 1
    "small": dict(size=512, seed=0, kind="affine", n_neighbors=1, psize=7, dim_reduced=8, leaf_size=32),
    # 1024x1024 version of the large pair (same generator and parameters): bounded profiler captures
    "medium": dict(size=1024, seed=1, kind="flow", n_neighbors=4, psize=9, dim_reduced=16, leaf_size=64),
}
# graph workloads (the parallel form under one CUDA graph launch per batch)
GRAPH_WORKLOADS = {
    # 64 pairs, sides U(256,1536), aspect U(0.5,2), random affine (seed 2): patch 7, PCA 8, k 1,
    # leaf size and passes autotuned per size class, all pairs in one graph launch
    "batch": dict(psize=7, dim_reduced=8, n_neighbors=1, leaf="auto", iters="auto", precision="bf16"),
    # 120 frames 1920x1080, each the previous warped (sigma 96, magnitude 6) + N(0,3^2) (seed 3):
    # consecutive pairs, patch 5, PCA 12, leaf 32, k 8, FP16 leaf tiles, learned proposals,
    # 8 pairs per graph launch
    "stream": dict(psize=5, dim_reduced=12, n_neighbors=8, leaf=32, iters=2, precision="fp16", per_graph=8),
}
L2_FLUSH_BYTES = 256 << 20
# the arithmetic each form computes in
DTYPES = {"plain": "f32", "openclopt": "f32", "parallel": "bf16", "learned": "bf16"}
ARITHMETIC = {
    "plain": "u8 images; FP64 covariance and eigendecomposition; exact FP32 projection; FP32 tree and "
             "leaf distances (no FMA, the reference's order); int32 raw-patch re-rank",
    "openclopt": "u8 images; FP64 covariance and eigendecomposition; exact FP32 projection; FP32 tree (median "
                 "of two middle values) and leaf distances; squared raw-patch re-rank",
    "parallel": "u8 images; FP64 covariance and Rayleigh-Ritz, FP32 subspace iteration; FP16 tensor-core "
                "projection (FP32 accumulate); FP32 tree; BF16 hi/lo tensor-core leaf tiles (FP32 accumulate) "
                "with an exact FP32 re-rank; int32 exact raw-patch SSD for every candidate",
}
ARITHMETIC["learned"] = ARITHMETIC["parallel"] + "; BF16 tensor-core proposal network (FP32 accumulate)"


def make_pair(w):
    from annfmp_gb300 import gen
    if w["kind"] == "flow":
        return gen.pair_flow(w["seed"], w["size"])
    return gen.pair_small(w["seed"], w["size"])


def params_of(w):
    n_b = (w["size"] - w["psize"] + 1) ** 2
    return dict(n_neighbors=w["n_neighbors"], psize=w["psize"], dim_reduced=w["dim_reduced"],
                n_subset=int(round(0.1 * n_b)), leaf_size=w["leaf_size"], seed=w["seed"])


# ---------------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()  # the timed region starts once sampling runs
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# algorithmic bytes of each stage per NNF: the bytes the algorithm touches (served by DRAM, L2 or
# L1), the numerator of the roofline's achieved bandwidth
# ---------------------------------------------------------------------------------------------
def stage_bytes(stage, w, n_a, n_b, depth, n_cols, it=1, nrand=1, n_prop=0, count=1):
    """Algorithmic bytes of one stage per NNF (count = how many times the stage's mark repeats
    in one fit, e.g. the global tree levels)."""
    d, k, P = w["dim_reduced"], w["n_neighbors"], w["psize"] ** 2 * 3
    ppl = n_b / float(1 << depth)
    rows_q = n_a - n_cols
    n_sub = int(round(0.1 * n_b))
    if stage == "chain":  # per query: query + k propagated leaves + leaf spans + natural list + k-list out
        return rows_q * (4 * d + k * ppl * 4 * d + 8 * k + 12 * k + 4 * k)
    if stage == "natural_knn":  # tensor-core tiles: every leaf's points staged once, each query in, list out
        return n_b * 4 * d + n_a * (4 * d + 4 + 4 * k)
    if stage == "natural_leaf":  # query + node path + leaf id out
        return n_a * (4 * d + 8 * depth + 4)
    if stage == "next_range":  # per tree position: its row-below position's leaf span
        return n_b * (4 + 4 + 8)
    if stage == "tc_group":  # query + node path + leaf id, then the leaf-ordered query list
        return n_a * (4 * d + 8 * depth + 4 + 8)
    if stage == "fast_init":  # k candidate positions + proposals + A patch + k + n_prop B patches + match out
        return n_a * (4 * k + 4 * n_prop + (k + n_prop + 1) * P + 8)
    if stage == "fast_propagate":  # per pass: match in/out, 4 neighbour matches, A patch, 4 + nrand B patches
        return n_a * (8 + 16 + (5 + nrand) * P + 8) * max(it, 1)
    if stage == "select_best":  # k A/B patch pairs + list in + index/distance out
        return n_a * (k * 2 * P + 4 * k + 8)
    if stage == "first_row":  # every point once per 128-query tile
        return -(-n_cols // 128) * n_b * 4 * d + n_cols * 4 * d
    if stage == "project":  # both images: pixels in, reduced patches out
        return 2 * ((w["size"] ** 2) * 3 + n_b * 4 * d)
    if stage == "build_level":  # per global level and point: split coordinate in, key out, two more
        # digit passes and the count over the keys, the scatter's key, row and index in and out
        return count * n_b * (4 + 4 + 4 + 4 + 4 + (4 + 4 * d + 4) + (4 * d + 4))
    if stage == "build_subtree":  # rows and indices in and out once, point leaf out, leaf boxes
        return n_b * (2 * (4 * d + 4) + 4) + (1 << depth) * 2 * 4 * d
    if stage == "pca_gram":  # sampled patches gathered from the images, written blocked, read by the Gram
        return 3 * n_sub * P
    if stage == "pca_eigh":  # the covariance in, the components out (latency-bound)
        return 8 * P * P + 8 * d * P
    return None


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


# ---------------------------------------------------------------------------------------------
# CPU arm (oracle)
# ---------------------------------------------------------------------------------------------
def _transform(O, patches, comps, mean, chunk=262144):
    """The reference's FP64 projection, in chunks (bounded host memory)."""
    return np.concatenate([O.pca_transform(patches[i:i + chunk], comps, mean) for i in range(0, len(patches), chunk)])


def cpu_full(a, b, w):
    """Time the oracle's complete plain-method fit of the pair (annfmp/openmp/base.py:53-150):
    PCA fit, extraction and projection of both images, tree, and the whole row loop (first row,
    every later row, re-rank). Returns (seconds, per-stage detail, NNF)."""
    from oracle import oracle as O
    prm = params_of(w)
    p = w["psize"]
    n_rows, n_cols = a.shape[0] - p + 1, a.shape[1] - p + 1
    t0 = time.perf_counter()
    comps, mean = O.pca_fit(a, b, p, prm["dim_reduced"], prm["n_subset"], prm["seed"])
    t1 = time.perf_counter()
    pb = O.extract_patches(b, p)
    bred = _transform(O, pb, comps, mean)
    pa = O.extract_patches(a, p)
    ared = _transform(O, pa, comps, mean)
    t2 = time.perf_counter()
    tree = O.OracleTree(bred, O.tree_depth(len(bred), prm["leaf_size"]))
    t3 = time.perf_counter()
    final, _ = tree.process_rows(ared, pa, pb, n_rows, n_cols, prm["n_neighbors"])
    t4 = time.perf_counter()
    det = dict(pca_fit=round(t1 - t0, 3), patches_and_projection=round(t2 - t1, 3), tree=round(t3 - t2, 3),
               rows=round(t4 - t3, 3))
    return t4 - t0, det, final


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


def run_reference(args, w, rank, world):
    if rank != 0:
        return
    a, b = make_pair(w)
    p = w["psize"]
    n_a = (a.shape[0] - p + 1) * (a.shape[1] - p + 1)
    for _ in range(args.warmup):
        cpu_full(a, b, w)
    times = []
    for _ in range(args.steps):
        t, det, _ = cpu_full(a, b, w)
        times.append(t)
    t = float(np.mean(times))
    cores = cpu_threads()
    val = n_a / t
    line = {"metric": "query patches/s", "value": val, "unit": "query patches/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "form": "plain", "config": config_of(w, args),
            "cpu_baseline": {"value": val, "unit": "query patches/s", "cores": cores, "kind": "port",
                             "sample": f"every step one complete plain-method fit of the pair by the oracle (C "
                                       f"restatement, OpenMP over {cores} threads, numpy PCA): all {n_a} query "
                                       f"patches, nothing extrapolated (last step: {det})"},
            "e2e": {"value": val, "unit": "query patches/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(w, args):
    """The workload, identical in both arms (the form each arm runs is a key of its own)."""
    prm = params_of(w)
    return {"workload": f"{w['size']}x{w['size']}x3 {w['kind']} pair seed {w['seed']}, patch {w['psize']}x"
                        f"{w['psize']}x3, PCA {w['dim_reduced']}, leaf {w['leaf_size']}, k {w['n_neighbors']}",
            "n_subset": prm["n_subset"], "pairs_per_rank": 1,
            "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{args.gpus}"}


# ---------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------
def reduce_max(x: float, world: int, device=None) -> float:
    """The slowest rank's value (max over ranks; a no-op for one rank). Works with NCCL on CUDA
    tensors and with gloo on CPU tensors."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: int, ms: float, world: int) -> float:
    """Whole-job throughput of `world` replicas that each processed units_per_rank in the slowest
    rank's time ms (weak scaling, no data-path collective)."""
    return world * units_per_rank / (ms / 1e3)


def learned_available():
    from annfmp_gb300.proposal import DEFAULT_WEIGHTS
    return os.path.exists(DEFAULT_WEIGHTS)


def make_model(form, args, prm, local_rank, graph="auto"):
    """plain: the reference's method; parallel: subspace PCA, BF16 tensor-core projection and leaf
    tiles, parallel propagation; learned: parallel + the trained offset-proposal network. The
    parallel forms replay a captured CUDA graph from their third fit on (graph="auto")."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    if form == "openclopt":  # the reference GPU backend's algorithm (K 8), eager
        from annfmp_gb300 import ANNFieldPropKDTreeOpenCLOPTGB300
        return ANNFieldPropKDTreeOpenCLOPTGB300(psize=prm["psize"], dim_reduced=prm["dim_reduced"],
                                                n_subset=prm["n_subset"], leaf_size=prm["leaf_size"],
                                                seed=prm["seed"], verbose=0, device_id=local_rank)
    kw = dict(verbose=0, device=local_rank, graph=graph, **prm)
    if form == "plain":
        return ANNFieldPropKDTreeGB300(**kw)
    proposal = None
    if form == "learned":
        from annfmp_gb300.proposal import ProposalNet
        proposal = ProposalNet.pretrained(local_rank)
    return ANNFieldPropKDTreeGB300(form="parallel", iters=args.iters, proposal=proposal, **kw)


def time_form(form, args, prm, local_rank, A, B, flush, steps):
    """(ms per step, last NNF) of a form on device-resident images, CUDA events, L2 flushed."""
    import torch
    model = make_model(form, args, prm, local_rank)
    for _ in range(max(args.warmup, 1)):
        model.fit(A, B)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        evs[i][0].record()
        nn = model.fit(A, B)
        evs[i][1].record()
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in evs) / steps, nn


def run_gpu(args, w, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from annfmp_gb300 import ANNFieldPropKDTreeGB300, _lib
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    a, b = make_pair(w)
    prm = params_of(w)
    p = w["psize"]
    n_rows, n_cols = a.shape[0] - p + 1, a.shape[1] - p + 1
    n_a = n_rows * n_cols
    n_b = (b.shape[0] - p + 1) * (b.shape[1] - p + 1)
    A = torch.from_numpy(a).to(dev)
    B = torch.from_numpy(b).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    model = make_model(args.form, args, prm, local_rank)

    for _ in range(args.warmup):
        model.fit(A, B)
    torch.cuda.synchronize(dev)
    graphed = getattr(model, "_graph", None) is not None
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    launches0 = _lib.launch_count()
    with ClockSampler(dev.index) as clocks:
        t_wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record()
            nn_dev = model.fit(A, B)
            ev[i][1].record()
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall0
    launches = _lib.launch_count() - launches0
    if graphed:  # a replay launches the kernels the capture recorded
        launches = args.steps * model._graph["kernels"]
    ms = reduce_max(sum(s.elapsed_time(e) for s, e in ev) / args.steps, world, dev)

    # per-stage kernel times: the same form run eagerly with the library's stage marks
    pm = make_model(args.form, args, prm, local_rank, graph=False)
    pm.fit(A, B)
    h = pm.kdtree.handle
    h.profile(True)
    h.profile_read(torch.cuda.current_stream(dev).cuda_stream)
    stages = {}
    stage_counts = {}
    for i in range(max(2, min(args.steps, 4))):
        flush.fill_(float(i))
        pm.fit(A, B)
        step = {}  # a stage that repeats within a fit (per image, per tree level) adds up
        counts = {}
        for name, sms in h.profile_read(torch.cuda.current_stream(dev).cuda_stream):
            step[name] = step.get(name, 0.0) + sms
            counts[name] = counts.get(name, 0) + 1
        stage_counts = counts
        for name, sms in step.items():
            stages.setdefault(name, []).append(sms)
    h.profile(False)
    if world > 1:
        dist.barrier()

    # end to end through the public API: pinned host images in, host NNF out
    a_pin = torch.from_numpy(a).pin_memory()
    b_pin = torch.from_numpy(b).pin_memory()
    e2e_times = []
    for i in range(max(2, args.steps)):
        flush.fill_(float(i))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        nn = model.fit(a_pin, b_pin)
        nn_host = nn.cpu()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = reduce_max(float(np.median(e2e_times)), world, dev)

    if rank != 0:
        return
    stage_ms = {k: float(np.mean(v)) for k, v in stages.items()}
    kernel_stages = {k: v for k, v in stage_ms.items() if not k.endswith(":begin")}
    depth = pm.kdtree.final_tree_depth_
    peak, peak_kind = load_peaks()
    # proposals with a seed method are verified on their own handle beside the PCA fit: the
    # profiled fast_init then reads one seed match per pixel, not the proposals
    prop_src = getattr(pm, "proposal", None)
    n_prop = 0 if prop_src is None or hasattr(prop_src, "seed") else int(getattr(prop_src, "per_pixel", 4))
    search = getattr(pm, "search", (1, 2))

    def sb(k):
        return stage_bytes(k, w, n_a, n_b, depth, n_cols, args.iters, search[0], n_prop, stage_counts.get(k, 1))
    # the dominant stage: the largest of ALL stages (every stage has a byte model)
    dom = max(kernel_stages, key=lambda k: kernel_stages[k])
    by = sb(dom) or 0
    # distance error of the last timed NNF against the exact raw-patch nearest neighbour
    from annfmp_gb300 import metrics
    quality = metrics.distance_ratio_error(a, b, nn_dev, p, n_samples=4096, seed=w["seed"] + 7, device=local_rank)
    # the other forms on the same pair, same timing rules (for the speed-up at equal error)
    forms = {args.form: {"ms_per_step": ms, "value": n_a / (ms / 1e3), "distance_error": quality}}
    if world == 1 and not args.no_compare:
        for f in ("plain", "parallel", "learned", "openclopt"):
            if f == args.form or (f == "learned" and not learned_available()):
                continue
            fms, fnn = time_form(f, args, prm, local_rank, A, B, flush, max(2, args.steps // 2))
            fq = metrics.distance_ratio_error(a, b, fnn, p, n_samples=4096, seed=w["seed"] + 7, device=local_rank)
            forms[f] = {"ms_per_step": fms, "value": n_a / (fms / 1e3), "distance_error": fq}
    achieved = by / (kernel_stages[dom] / 1e3) / 1e9
    traffic = load_traffic().get(f"{args.workload}:{args.form}:{dom}")
    value = replica_value(n_a, ms, world)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "algorithmic_bytes": by, "per": "NNF (all launches of the stage)",
            "traffic": traffic}
    if traffic:  # what DRAM itself delivered (ncu capture of the same stage), beside the touched bytes
        roof["dram_achieved"] = traffic / (kernel_stages[dom] / 1e3) / 1e9
        roof["dram_frac"] = roof["dram_achieved"] / peak
    if dom in BINDING:
        roof["binding_unit"], roof["binding_evidence"] = BINDING[dom]
    line = {
        "metric": "query patches/s", "value": value, "unit": "query patches/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.form], "arithmetic": ARITHMETIC[args.form], "data": "synthetic",
        "form": args.form, "iters": args.iters if args.form != "plain" else None,
        "execution": "one CUDA graph replay per NNF" if graphed else "eager",
        "config": config_of(w, args),
        "e2e": {"value": replica_value(n_a, e2e_s * 1e3, world), "unit": "query patches/s",
                "h2d_bytes_per_step": int(a.nbytes + b.nbytes),
                "d2h_bytes_per_step": int(nn_host.numel() * nn_host.element_size())},
        "gpu_launches": int(launches),
        "roofline": roof,
        # per stage: algorithmic bytes over the HBM copy peak, and the unit ncu found binding (a
        # stage bound elsewhere, e.g. L1, can show an HBM fraction above 1.0: its bytes come from
        # L1/L2, so that fraction is not a bandwidth result)
        "roofline_stages": {k: {"ms": v, "algorithmic_bytes": sb(k), "frac": (sb(k) or 0) / (v / 1e3) / 1e9 / peak,
                                "bound": BINDING[k][0] if k in BINDING else "hbm"}
                            for k, v in sorted(kernel_stages.items(), key=lambda kv: -kv[1])},
        "distance_error": quality,
        "forms": forms,
        "stages_ms": stage_ms, "stage_marks_per_fit": stage_counts, "wall_ms_per_step": t_wall * 1e3 / args.steps,
        "clocks": clocks.summary(),
    }
    if world == 1 and not args.no_cpu_baseline:
        t_cpu, det, _ = cpu_full(a, b, w)
        line["cpu_baseline"] = {"value": n_a / t_cpu, "unit": "query patches/s", "cores": cpu_threads(),
                                "kind": "port", "sample": f"one complete plain-method fit of the pair by the oracle "
                                                          f"(all {n_a} query patches, nothing extrapolated; {det})"}
    if world == 1 and not args.no_compare:
        del model, pm
        torch.cuda.empty_cache()
        line["workloads"] = other_workloads(args, local_rank, flush)
    print(json.dumps(line), flush=True)


# where ncu located the binding unit of a stage's main kernel (committed summaries)
BINDING = {
    "fast_propagate": ("l1", "profiles/fast_prop_t_kernel_medium_learned.md: L1 throughput 88% in pass 1, DRAM < 2%"),
    "fast_init": ("l1", "profiles/fast_init_t_kernel_medium_learned.md: L1 throughput 91%, DRAM 2%"),
    "natural_knn": ("issue (per-query selection and exact re-rank)",
                    "profiles/leaf_tc_kernel_medium_learned.md: tensor pipe 3.5%, 16 warps per SM (TMEM limit)"),
    "build_subtree": ("barrier", "profiles/subtree_kernel_medium_learned.md: barrier stalls 4.0 per issue"),
    "chain": ("latency (dependent loads per row step; 20.3 GB of DRAM re-reads per fit)",
              "profiles/chain_sel_kernel_medium_plain.md, profiles/dram_large_plain.md"),
}


def other_workloads(args, local_rank, flush):
    """The 512x512 pair by the plain method (with the oracle on the same pair), the 64 uneven
    pairs in one graph launch and the 1920x1080 frame stream: each timed with its own events
    and checked for distance error, so one default run records every workload."""
    from annfmp_gb300 import metrics
    import torch
    out = {}
    w = WORKLOADS["small"]
    a, b = make_pair(w)
    prm = params_of(w)
    p = w["psize"]
    n_a = (a.shape[0] - p + 1) * (a.shape[1] - p + 1)
    dev = torch.device("cuda", local_rank)
    A, B = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    rec = {"config": config_of(w, args)}
    for f in ("plain", "learned" if learned_available() else "parallel"):
        fms, fnn = time_form(f, args, prm, local_rank, A, B, flush, max(3, args.steps // 2))
        rec[f] = {"ms_per_step": fms, "value": n_a / (fms / 1e3),
                  "distance_error": metrics.distance_ratio_error(a, b, fnn, p, n_samples=4096, seed=w["seed"] + 7,
                                                                 device=local_rank)}
        if f == "plain":
            nn_plain = fnn.cpu().numpy()
    t_cpu, det, nn_cpu = cpu_full(a, b, w)
    rec["cpu_oracle"] = {"ms_per_step": t_cpu * 1e3, "value": n_a / t_cpu, "cores": cpu_threads(), "detail": det}
    rec["plain_nnf_identical_to_oracle"] = float((nn_plain == nn_cpu).mean())
    out["small"] = rec
    gargs = argparse.Namespace(**vars(args))
    gargs.steps = 3
    for name in ("batch", "stream"):
        out[name] = run_graph_workload(gargs, name, 0, 1, local_rank, emit=False)
        torch.cuda.empty_cache()
    return out


def run_graph_workload(args, name, rank, world, local_rank, emit=True):
    """Batched pairs under CUDA graphs: value = query patches of all pairs / time of the launches.
    Prints the JSON line (emit) or returns it."""
    import torch

    from annfmp_gb300 import _lib, gen
    from annfmp_gb300.batch import Autotuner, BatchNNF
    cfg = GRAPH_WORKLOADS[name]
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    kw = dict(n_neighbors=cfg["n_neighbors"], psize=cfg["psize"], dim_reduced=cfg["dim_reduced"],
              leaf_precision=cfg["precision"], seed=0, device=local_rank)
    p = cfg["psize"]
    if name == "batch":
        pairs = gen.gpu_pairs_uneven(2, 64, device=local_rank)
        t0 = time.perf_counter()
        groups = [BatchNNF(leaf_size=cfg["leaf"], iters=cfg["iters"], tuner=Autotuner(max_error=0.005, samples=512, reps=1),
                           **kw).prepare(pairs)]
        t_prep = time.perf_counter() - t0
        feeds = [None]
    else:
        from annfmp_gb300.proposal import ProposalNet
        frames = gen.gpu_frame_stream(3, 120, 1080, 1920, device=local_rank)
        pairs = [(frames[i], frames[i + 1]) for i in range(len(frames) - 1)]
        per = cfg["per_graph"]
        chunks = [pairs[i:i + per] for i in range(0, len(pairs), per)]
        t0 = time.perf_counter()
        prop = ProposalNet.pretrained(local_rank) if learned_available() else None
        groups = [BatchNNF(leaf_size=cfg["leaf"], iters=cfg["iters"], proposal=prop, **kw).prepare(chunks[0])]
        if len(chunks[-1]) != per:
            groups.append(BatchNNF(leaf_size=cfg["leaf"], iters=cfg["iters"], proposal=prop, **kw).prepare(chunks[-1]))
        t_prep = time.perf_counter() - t0
        feeds = chunks
    n_a = sum((a.shape[0] - p + 1) * (a.shape[1] - p + 1) for a, _ in pairs)

    def one_pass():
        if name == "batch":
            groups[0].run()
            return
        for ch in feeds:  # copy each batch of frame pairs into the graph's inputs, then one launch
            bt = groups[0] if len(ch) == cfg["per_graph"] else groups[-1]
            for (A, B), (a, b) in zip(bt.inputs, ch):
                A.copy_(a)
                B.copy_(b)
            bt.run()

    for _ in range(max(args.warmup, 1)):
        one_pass()
    torch.cuda.synchronize(dev)
    # kernels per timed step: graph replays launch the kernels captured in them
    per_step = sum(groups[0 if (name == "batch" or len(ch) == cfg["per_graph"]) else -1].kernels_per_launch
                   for ch in feeds)
    launches0 = _lib.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(dev.index) as clocks:
        for i in range(args.steps):
            ev[i][0].record()
            one_pass()
            ev[i][1].record()
        torch.cuda.synchronize(dev)
    ms = reduce_max(sum(a.elapsed_time(b) for a, b in ev) / args.steps, world, dev)
    # a sample of pairs checked against the exact raw-patch nearest neighbour
    from annfmp_gb300 import metrics
    errs = []
    if name == "batch":
        outs = groups[0].run()
        torch.cuda.synchronize(dev)
        for i in range(0, len(pairs), 16):
            errs.append(metrics.distance_ratio_error(pairs[i][0], pairs[i][1], outs[i], p, n_samples=1024, seed=9,
                                                     device=local_rank)["mean"])
    else:
        bt = groups[0]
        for (A, B), (a, b) in zip(bt.inputs, feeds[0]):
            A.copy_(a)
            B.copy_(b)
        outs = bt.run()
        torch.cuda.synchronize(dev)
        for i in (0, len(outs) - 1):
            errs.append(metrics.distance_ratio_error(bt.inputs[i][0], bt.inputs[i][1], outs[i], p, n_samples=1024,
                                                     seed=9, device=local_rank)["mean"])
    if rank != 0:
        return
    settings = sorted(set(tuple(x) for g in groups for x in g.settings()))
    line = {
        "metric": "query patches/s", "value": replica_value(n_a, ms, world), "unit": "query patches/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": cfg["precision"], "data": "synthetic (generated on the GPU)",
        "config": {"workload": name, "pairs": len(pairs), "psize": p, "dim_reduced": cfg["dim_reduced"],
                   "k": cfg["n_neighbors"], "leaf_iters_chosen": settings, "graphs_per_step": len(feeds),
                   "form": "parallel" + ("+learned" if name == "stream" and learned_available() else ""),
                   "l2": "inputs of the whole pass exceed L2"},
        "distance_error_mean_sampled_pairs": errs, "prepare_s": t_prep,
        "gpu_launches": int(_lib.launch_count() - launches0) + per_step * args.steps,
        "graph_launches_per_step": len(feeds), "clocks": clocks.summary(),
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS) + sorted(GRAPH_WORKLOADS))
    ap.add_argument("--form", default="learned", choices=["plain", "parallel", "learned", "openclopt"],
                    help="plain: the reference's method; parallel: BF16 tensor-core form; learned: + proposals; "
                         "openclopt: the reference GPU backend's algorithm")
    ap.add_argument("--iters", type=int, default=3, help="propagation passes of the parallel forms")
    ap.add_argument("--no-compare", action="store_true", help="time only --form (not the other forms)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.workload in GRAPH_WORKLOADS:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "graph workloads have no CPU counterpart"}))
            return
        run_graph_workload(args, args.workload, int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
                           int(os.environ.get("LOCAL_RANK", 0)))
        return
    w = WORKLOADS[args.workload]
    if args.form == "learned" and not learned_available():
        print("bench: no trained proposal weights; timing the parallel form", file=sys.stderr)
        args.form = "parallel"
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, w, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("ANNF_PG", "nccl") == "nccl" else "gloo")
    try:
        run_gpu(args, w, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
