#!/usr/bin/env python
"""Benchmark of the embedding hot path: normalize_cells (both copies) ->
scale_features (3,000 features, implicit centre/scale/clip) -> irlba PCA (50)
-> kNN (20), on one GB300, with counts already resident in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload atlas|plain|small] [--cells N] [--batched] [--reader]
                    [--kernel-case irlba|knn] [--accuracy-study] [--no-e2e] [--no-fp32]
                    [--no-cpu] [--no-accuracy] [--no-knn-stress]

Prints one JSON line (rank 0).  Workload "atlas": 1,300,000 cells x 27,998
genes, ~2,000 non-zeros per cell, 40 latent clusters, values stored in BF16
with FP32 product accumulation and FP64 Lanczos reorthogonalisation/restart.
The plain-FP32 form of the same pipeline is timed on the same data for the
mixed-vs-FP32 ratio.  Data: seeded synthetic negative-binomial counts (no
public dataset is read).  --impl reference times the CPU oracle (the
restatement of the reference's CPU path) on a bounded sample.  --batched runs
the batched-samples workload (64 samples of 500-50,000 cells: one launch per
stage for all samples against one sample after another); --reader times the
MatrixMarket reader (text in host memory to the device count matrix);
--kernel-case runs one small case of a kernel family for profiler captures.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("cells/s norm→PCA50→kNN20 @1.3M: mixed vs FP32 on GB300 (σ err≤1e-4); "
          "SpMM HBM%")

WORKLOADS = {
    # 1.3M-cell atlas, mixed precision (the configuration the metric is quoted on)
    "atlas": dict(n_cells=1_300_000, n_genes=27_998, mu_mean=-1.2, mu_sd=1.6, nnz_per_cell=2000,
                  n_clusters=40, n_hvf=3000, npcs=50, k=20, dtype="bfloat16", knn="bf16"),
    # 100k cells x 33,538 genes, plain FP32
    "plain": dict(n_cells=100_000, n_genes=33_538, mu_mean=-1.2, mu_sd=1.6, nnz_per_cell=2500,
                  n_clusters=0, n_hvf=3000, npcs=50, k=20, dtype="float32", knn="fp32"),
    # the CPU-runnable reference case
    "small": dict(n_cells=2_000, n_genes=20_000, mu_mean=-1.0, mu_sd=1.5, nnz_per_cell=1000,
                  n_clusters=0, n_hvf=2000, npcs=50, k=20, dtype="float64", knn="fp32"),
}
# batched samples: many samples of different sizes through one launch per stage
BATCHED = dict(n_samples=64, n_genes=20_000, cells_min=500, cells_max=50_000, depth_sd=0.5,
               mu_mean=-1.2, mu_sd=1.6, nnz_per_cell=1000, n_clusters=10, n_hvf=2000, npcs=30,
               k=15, dtype="bfloat16", knn="bf16")
SEED = 20261203
# DRAM bytes per algorithmic byte of the X v product kernel, from an ncu capture
# of the 100,000-cell case (425.1 + 4.1 MB read + written for 425.7 MB algorithmic)
SPMV_TRAFFIC_PER_BYTE = 429.2 / 425.7
SCALE_FACTOR = 1e4
SCALE_MAX = 10.0
DISPERSION = 0.2
# CPU baseline samples (cells): the baseline leg of this arm, and the reference arm
CPU_BASELINE_SIZES = (16_250, 65_000)
REF_LARGE, REF_SMALL, REF_WARM = 130_000, 32_500, 2_000


# ---------------------------------------------------------------------------
# synthetic parameters
# ---------------------------------------------------------------------------
def gen_params(w, n_cells, seed):
    rng = np.random.default_rng(seed)
    g = w["n_genes"]
    mu_g = rng.lognormal(w["mu_mean"], w["mu_sd"], g)
    s_c = rng.lognormal(0.0, 0.3, n_cells)
    cl = lfc = None
    if w["n_clusters"]:
        cl = rng.integers(0, w["n_clusters"], n_cells).astype(np.int32)
        lfc = np.zeros((w["n_clusters"], g), dtype=np.float32)
        for c in range(w["n_clusters"]):
            sel = rng.random(g) < 0.05
            lfc[c, sel] = rng.normal(0.0, 0.8, sel.sum())
    return mu_g, s_c, cl, lfc


def calibrate_depth(mu_g, s_c, cl, lfc, target, phi=DISPERSION, sample=256, seed=1):
    """Depth factor D with E[non-zeros per cell] = target under the NB model."""
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(s_c), min(sample, len(s_c)), replace=False)
    base = s_c[idx, None] * mu_g[None, :]
    if cl is not None:
        base = base * np.exp(lfc[cl[idx]])

    def nnz(D):
        m = D * base
        return float(np.mean(np.sum(1.0 - (1.0 + phi * m) ** (-1.0 / phi), axis=1)))

    lo, hi = 1e-4, 1e3
    for _ in range(36):
        mid = math.sqrt(lo * hi)
        if nnz(mid) < target:
            lo = mid
        else:
            hi = mid
    return math.sqrt(lo * hi)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# distributed helpers (replicas: one independent pipeline per GPU)
# ---------------------------------------------------------------------------
def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        return td, td.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def barrier(td):
    if td is not None:
        td.barrier()


def allmax(td, x):
    if td is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# the GPU pipeline
# ---------------------------------------------------------------------------
def run_pipeline(sv, ctx, counts, hvf, w, init, form, marks=False):
    """One step: normalise -> scale -> PCA -> kNN on device-resident counts.
    form: (value dtype, knn precision).  Returns (embedding, knn handle)."""
    dtype, knn = form
    if marks:
        ctx.mark(1)
    d = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=dtype, ctx=ctx)
    if marks:
        ctx.mark(2)
    S = sv.scale_features(d, scale_max=SCALE_MAX, features=hvf)
    if marks:
        ctx.mark(3)
    em = sv.pca(S, w["npcs"], tol=1e-5, init=init, download=False)
    if marks:
        ctx.mark(4)
    _, _, kh = sv.ann(em, w["k"], precision=knn, ctx=ctx, keep=True, download=False)
    if marks:
        ctx.mark(5)
    return d, S, em, kh


def timed_steps(sv, ctx, td, counts, hvf, w, init, form, steps, warmup, with_stages=False):
    for _ in range(warmup):
        run_pipeline(sv, ctx, counts, hvf, w, init, form)
    ctx.sync()
    barrier(td)
    stages = {"normalize": 0.0, "scale": 0.0, "pca": 0.0, "knn": 0.0}
    l0 = ctx.launches()
    t0 = time.perf_counter()
    ctx.mark(0)
    info = None
    for _ in range(steps):
        d, S, em, kh = run_pipeline(sv, ctx, counts, hvf, w, init, form, marks=with_stages)
        if with_stages:
            ctx.sync()
            stages["normalize"] += ctx.elapsed_ms(1, 2)
            stages["scale"] += ctx.elapsed_ms(2, 3)
            stages["pca"] += ctx.elapsed_ms(3, 4)
            stages["knn"] += ctx.elapsed_ms(4, 5)
        info = em.info
        del d, S, em, kh
    ctx.mark(6)
    ctx.sync()
    wall = time.perf_counter() - t0
    dev_ms = ctx.elapsed_ms(0, 6)
    launches = ctx.launches() - l0
    barrier(td)
    return {"dev_ms": dev_ms, "wall_s": wall, "launches": launches,
            "stages_ms": {k: v / steps for k, v in stages.items()} if with_stages else None,
            "irlba": info}


def snn_stage(sv, ctx, counts, hvf, w, init, form, reps=3):
    """shared_nearest_neighbours timed on its own (src/neighbours.jl:76-108,
    272-278): the Jaccard graph of the step's kNN lists (k, prune 1/15, in the
    coordinates' FP64 type) built on the device, CUDA events around the call,
    best of `reps`.  Bytes: the kNN lists read (4 n k), the reverse lists
    written and read (8 n k), the graph written (12 nnz + 8 (n + 1))."""
    import ctypes as C
    _, _, em, kh = run_pipeline(sv, ctx, counts, hvf, w, init, form)
    lib = sv._lib.load()
    best, nnz = None, 0
    for _ in range(reps):
        h = C.c_void_p()
        ctx.sync()
        ctx.mark(7)
        sv._lib.check(lib.sv_snn_knn(ctx.h, kh.h, int(w["k"]), 1.0 / 15.0, sv._lib.SV_F64, C.byref(h)))
        ctx.mark(8)
        ctx.sync()
        ms = ctx.elapsed_ms(7, 8)
        g = sv.Graph(ctx, h)
        a, b = C.c_int64(), C.c_int64()
        sv._lib.check(lib.sv_graph_info(h, C.byref(a), C.byref(b)))
        nnz = b.value
        del g
        best = ms if best is None else min(best, ms)
    n, k = w["n_cells"], w["k"]
    byts = 4 * n * k + 8 * n * k + 12 * nnz + 8 * (n + 1)
    return {"ms": round(best, 3), "nnz": int(nnz), "edges_per_cell": round(nnz / n, 2),
            "bytes": int(byts), "gbs": round(byts / (best / 1e3) / 1e9, 1)}


def e2e_steps(sv, ctx, td, host, shape, hvf, w, init, form, steps, outs=None):
    """The same pipeline through the public API with host buffers: upload of the
    CSC counts (pinned host memory) and download of Z, nn_index and distances
    (into the pinned arrays `outs` = (Z, nn_index, distances) when given)."""
    colptr, rowval, nzval = host
    Zo, io, do = outs if outs else (None, None, None)
    n = shape[0]
    h2d = colptr.nbytes + rowval.nbytes + nzval.nbytes
    d2h = 0
    ctx.sync()
    barrier(td)
    t0 = time.perf_counter()
    for _ in range(steps):
        counts = sv.CountMatrix.upload(colptr, rowval, nzval, shape, 0, ctx)
        d = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=form[0], ctx=ctx)
        S = sv.scale_features(d, scale_max=SCALE_MAX, features=hvf)
        em = sv.pca(S, w["npcs"], tol=1e-5, init=init, download=True, out=Zo)
        idx, dist = sv.ann(em, w["k"], precision=form[1], ctx=ctx,
                           out=(io, do) if io is not None else None)
        d2h = (em.coordinates.nbytes + em.stdev.nbytes + em.basis.nbytes + idx.nbytes + dist.nbytes)
        del counts, d, S, em
    ctx.sync()
    dt = time.perf_counter() - t0
    barrier(td)
    return dt, h2d, d2h


def pinned_copy(sv, arr):
    """Copies a numpy array into pinned host memory (sv_host_alloc)."""
    import ctypes as C
    lib = sv._lib.load()
    p = C.c_void_p()
    sv._lib.check(lib.sv_host_alloc(C.byref(p), max(1, arr.nbytes)))
    buf = (C.c_byte * max(1, arr.nbytes)).from_address(p.value)
    out = np.frombuffer(buf, dtype=arr.dtype, count=arr.size)
    out[:] = arr
    return out, p


def profile_step(sv, ctx, counts, hvf, w, init, form):
    """One extra step with per-kernel CUDA events (outside the timed steps)."""
    ctx.profile_reset()
    ctx.profile(True)
    run_pipeline(sv, ctx, counts, hvf, w, init, form)
    ctx.sync()
    rep = ctx.profile_report()
    ctx.profile(False)
    return rep


def roofline(rep, S_nnz, n_cells, n_hvf, dtype, peaks):
    """Roofline of the dominant HBM-bound kernel pair (the implicit SpMV)."""
    v = {"bfloat16": 2, "float32": 4, "float64": 8}[dtype]
    idx = 2 if n_hvf <= 65536 else 4
    # algorithmic bytes per launch: every stored entry (index + value) once, the
    # row pointers, and the input / output vectors
    csr = S_nnz * (idx + v) + 8 * (n_cells + 1) + 8 * n_cells
    csc = S_nnz * (4 + v) + 4 * n_cells
    out = {}
    for name, b in (("spmv_csr_h", csr), ("spmv_csc_chunks", csc)):
        if name in rep:
            cnt, ms = rep[name]
            avg = ms / cnt / 1e3
            out[name] = {"bytes": b, "avg_ms": avg * 1e3, "gbs": b / avg / 1e9, "launches": cnt}
    return out


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restatement of the reference's CPU path)
# ---------------------------------------------------------------------------
def cpu_params(w, n_cells, D=None):
    mu_g, s_c, cl, lfc = gen_params(w, n_cells, SEED)
    if D is None:
        D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
    return {"mu_g": mu_g, "s_c": s_c, "cluster": cl, "lfc": lfc, "depth": D, "dispersion": DISPERSION}


def cpu_model(recs, n_full):
    """Cells/s of the CPU path at n_full from two measured sample sizes: each
    stage's time grows as (n / n_large)^alpha with alpha measured between the
    two sizes (the PCA by its time per matrix product, at the large sample's
    product count).  Returns (cells/s, per-stage seconds at n_full, alphas)."""
    by_n = {}
    for r in recs:
        by_n.setdefault(r["n"], []).append(r)
    n1, n2 = sorted(by_n)[0], sorted(by_n)[-1]
    med = lambda rs, f: float(np.median([f(r) for r in rs]))
    out, alpha = {}, {}
    for st in ("normalize", "scale", "pca", "knn"):
        if st == "pca":
            f = lambda r: r["stages_s"]["pca"] / r["nmatvec"]
        else:
            f = lambda r, st=st: r["stages_s"][st]
        t1, t2 = med(by_n[n1], f), med(by_n[n2], f)
        a = math.log(t2 / t1) / math.log(n2 / n1) if t1 > 0 and t2 > 0 and n2 > n1 else 1.0
        a = min(max(a, 0.8), 2.5)
        alpha[st] = round(a, 3)
        t_full = t2 * (n_full / n2) ** a
        if st == "pca":
            t_full *= med(by_n[n2], lambda r: r["nmatvec"])
        out[st] = t_full
    return n_full / sum(out.values()), out, alpha


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="atlas", choices=sorted(WORKLOADS))
    ap.add_argument("--cells", type=int, default=0, help="override the cell count (smaller runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-knn-stress", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-samples and reader fields of the default atlas line")
    ap.add_argument("--kernel-case", choices=["irlba", "knn", "prep"], default=None,
                    help="run one small case of a kernel family (for profiler captures) and exit")
    ap.add_argument("--reader", action="store_true",
                    help="MatrixMarket reader: 10X-layout text in host memory to the device count matrix")
    ap.add_argument("--accuracy-study", action="store_true",
                    help="PC errors of every value type at two irlba tolerances (cause separation)")
    ap.add_argument("--batched", action="store_true",
                    help="the batched-samples workload (64 samples) instead of the atlas")
    args = ap.parse_args()
    if args.kernel_case:
        return kernel_case(args)
    if args.reader:
        return reader_bench(args)
    if args.batched:
        return batched_bench(args)
    if args.accuracy_study:
        return accuracy_study(args)
    w = dict(WORKLOADS[args.workload])
    if args.cells:
        w["n_cells"] = args.cells
    td, rank, world, local = dist_setup(args.gpus)

    if args.impl == "reference":
        return reference_arm(args, w, td, rank, world)

    import __graft_entry__ as ge
    ge._build_module().build()
    sv = ge.load_package()
    ctx = sv.Context(local)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)

    # ---- data (untimed): generated on the device ------------------------------
    n = w["n_cells"]
    mu_g, s_c, cl, lfc = gen_params(w, n, SEED + rank)
    D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
    t0 = time.perf_counter()
    counts = sv.CountMatrix.generate(n, w["n_genes"], mu_g, s_c, cl, lfc, depth=D,
                                     dispersion=DISPERSION, seed=SEED + rank, ctx=ctx)
    gen_s = time.perf_counter() - t0
    nnz = counts.nnz
    # HVF indices: a precomputed input (the reference selects them with vst,
    # src/variablefeatures.jl); stand-in: the most variable normalised genes
    d0 = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=w["dtype"], ctx=ctx)
    _, var = d0.gene_moments()
    hvf = np.sort(np.argsort(-var, kind="stable")[: w["n_hvf"]]) + 1
    del d0
    init = np.random.default_rng(SEED).standard_normal(w["n_hvf"])
    form = (w["dtype"], w["knn"])
    if form[1] == "bf16" and not knn_tc_available(sv, ctx):
        form = (form[0], "fp32")

    # ---- timed: device-resident -----------------------------------------------
    clk = ClockSampler(local)
    clk.start()
    res = timed_steps(sv, ctx, td, counts, hvf, w, init, form, args.steps, args.warmup)
    clocks = clk.stop()
    dev_ms = allmax(td, res["dev_ms"])
    ms_per_step = dev_ms / args.steps
    value = world * n * args.steps / (dev_ms / 1e3)

    # per-stage times (one extra pass with stage marks), per-kernel profile
    st = timed_steps(sv, ctx, None, counts, hvf, w, init, form, 1, 0, with_stages=True)
    snn = snn_stage(sv, ctx, counts, hvf, w, init, form)
    rep = profile_step(sv, ctx, counts, hvf, w, init, form)
    S = sv.scale_features(sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=w["dtype"],
                                             ctx=ctx), scale_max=SCALE_MAX, features=hvf)
    nnz_h = S.nnz
    del S
    rl = roofline(rep, nnz_h, n, w["n_hvf"], w["dtype"], peaks)
    top = sorted(rep.items(), key=lambda kv: -kv[1][1])[:8]

    # ---- plain FP32 form on the same data -----------------------------------
    fp32 = None
    if not args.no_fp32 and w["dtype"] != "float32":
        k32 = max(1, min(args.steps, 2))
        r32 = timed_steps(sv, ctx, td, counts, hvf, w, init, ("float32", "fp32"), k32, 1)
        ms32 = allmax(td, r32["dev_ms"]) / k32
        fp32 = {"value": world * n / (ms32 / 1e3), "ms_per_step": ms32, "steps": k32}

    # ---- accuracy against FP64 (untimed, rank 0) -------------------------------
    acc = None
    if rank == 0 and not args.no_accuracy:
        acc = accuracy(sv, ctx, counts, hvf, w, init, form)

    # ---- kNN stress case (untimed in the step; rank 0) ---------------------------
    stress = None
    if rank == 0 and not args.no_knn_stress and form[1] == "bf16":
        stress = knn_stress(sv, ctx, with_fp32=not args.no_fp32)

    # ---- e2e through the C ABI with host buffers ------------------------------
    e2e = None
    if not args.no_e2e:
        A = counts.to_csc()
        host = []
        keep = []
        for arr in (A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.astype(np.int32)):
            a, p = pinned_copy(sv, arr)
            host.append(a)
            keep.append(p)
        del A
        # results land in pinned host arrays allocated once, as the inputs do
        outs = []
        for shp, dt_ in (((n, w["npcs"]), np.float64), ((n, w["k"]), np.int32), ((n, w["k"]), np.float64)):
            a, p = pinned_copy(sv, np.zeros(shp[0] * shp[1], dtype=dt_))
            outs.append(a.reshape(shp, order="F"))
            keep.append(p)
        ke = max(1, min(args.steps, 3))
        e2e_steps(sv, ctx, td, host, (n, w["n_genes"]), hvf, w, init, form, 1, outs)   # warm-up
        dt, h2d, d2h = e2e_steps(sv, ctx, td, host, (n, w["n_genes"]), hvf, w, init, form, ke, outs)
        dt = allmax(td, dt)
        e2e = {"value": world * n * ke / dt, "unit": "cells/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": ke}
        lib = sv._lib.load()
        for p in keep:
            lib.sv_host_free(p)

    # ---- CPU baseline (rank 0, N = 1): the multi-threaded CPU restatement ------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import cpu_path
        sizes = [min(x, n) for x in CPU_BASELINE_SIZES]
        nt = cpu_path.threads()
        recs = cpu_path.run_in_subprocess(cpu_params(w, max(sizes), D), sizes, nt, seed=SEED,
                                          n_hvf=w["n_hvf"], npcs=w["npcs"], k=w["k"])
        val, st_full, alpha = cpu_model(recs, n)
        cpu = {"value": round(val, 2), "unit": "cells/s", "cores": nt, "kind": "port",
               "sample": (f"C/OpenMP restatement (FP64 products, numpy irlba over C basis "
                          f"operations, random-projection-tree kNN) on {sizes[0]} and {sizes[1]} cells of "
                          f"the same generator model on {nt} host threads; each stage extrapolated to "
                          f"{n} cells by its growth measured between the two sizes"),
               "stages_s_at_full": {k_: round(v, 2) for k_, v in st_full.items()},
               "growth_exponents": alpha,
               "knn_recall": recs[-1].get("knn_recall"),
               "measured": [{"n": r["n"], "stages_s": {k_: round(v, 3) for k_, v in r["stages_s"].items()},
                             "nmatvec": r["nmatvec"]} for r in recs]}

    if rank == 0:
        dom = max(rl.items(), key=lambda kv: kv[1]["avg_ms"] * kv[1]["launches"]) if rl else None
        roof = None
        if dom:
            name, r = dom
            roof = {"kernel": name, "bound": "hbm", "achieved": round(r["gbs"], 1),
                    "peak": hbm_peak, "unit": "GB/s", "frac": round(r["gbs"] / hbm_peak, 4),
                    "traffic": round(r["bytes"] * SPMV_TRAFFIC_PER_BYTE),
                    "traffic_source": "ncu dram__bytes_read+write of the same kernel on the 100,000-cell "
                                      "case, per algorithmic byte, scaled to this launch",
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                    "bytes_per_launch": r["bytes"], "avg_launch_ms": round(r["avg_ms"], 4)}
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": "cells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"bfloat16": "bf16", "float32": "f32", "float64": "f64"}[w["dtype"]],
            "data": "synthetic: seeded negative-binomial counts generated on the device (no dataset)",
            "config": {"workload": f"{args.workload}: {n} cells x {w['n_genes']} genes, "
                                   f"{nnz / n:.0f} nnz/cell, {w['n_hvf']} features, PCA {w['npcs']}, "
                                   f"kNN {w['k']}",
                       "n_cells": n, "n_genes": w["n_genes"], "nnz": nnz, "nnz_features": nnz_h,
                       "depth_factor": round(D, 5), "n_clusters": w["n_clusters"],
                       "value_dtype": w["dtype"], "knn_kernel": form[1],
                       "irlba": res["irlba"], "parallelism": f"replicas x{world}",
                       "l2": "inputs (tens of GB) exceed L2; no flush needed"},
            "stages_ms": st["stages_ms"],
            "snn": snn,
            "kernels_ms": {k: {"launches": c, "ms": round(ms, 3)} for k, (c, ms) in top},
            "spmv": rl,
            "roofline": roof,
            "e2e": e2e,
            "plain_fp32": fp32,
            "mixed_vs_fp32": round(fp32["ms_per_step"] / ms_per_step, 3) if fp32 else None,
            "cpu_baseline": cpu,
            "accuracy": acc,
            "knn_stress": stress,
            "gpu_launches": res["launches"],
            "clocks": clocks,
            "generate_s": round(gen_s, 2),
        }
        if world == 1 and args.workload == "atlas" and not args.cells and not args.no_extras:
            out.update(extras(args))
        print(json.dumps(out), flush=True)
    if td is not None:
        td.destroy_process_group()


def batched_bench(args, emit=True):
    """64 samples x 20,000 genes, cells per sample log-uniform in [500, 50,000],
    per-sample depth LogNormal(0, 0.5): normalise -> scale (per sample) -> PCA
    30 -> kNN 15 for every sample, (a) batched: one launch per stage over all
    samples (the Lanczos cycles of all samples in the same graph), (b) one
    sample after another through the single-sample calls.  Aggregate cells/s
    of both, on the same device-resident counts."""
    import __graft_entry__ as ge
    ge._build_module().build()
    sv = ge.load_package()
    ctx = sv.Context(0)
    w = dict(BATCHED)
    rng = np.random.default_rng(SEED + 4)
    sizes = np.exp(rng.uniform(np.log(w["cells_min"]), np.log(w["cells_max"]), w["n_samples"])).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    n = int(off[-1])
    mu_g, s_c, cl, lfc = gen_params(w, n, SEED + 4)
    depth = rng.lognormal(0.0, w["depth_sd"], w["n_samples"])
    s_c = s_c * np.repeat(depth, sizes)
    D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
    counts = sv.CountMatrix.generate(n, w["n_genes"], mu_g, s_c, cl, lfc, depth=D, dispersion=DISPERSION,
                                     seed=SEED + 4, ctx=ctx)
    d0 = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=w["dtype"], ctx=ctx)
    _, var = d0.gene_moments()
    hvf = np.sort(np.argsort(-var, kind="stable")[: w["n_hvf"]]) + 1
    del d0
    per = [counts.select_cells(int(off[i]), int(off[i + 1])) for i in range(w["n_samples"])]
    init = np.random.default_rng(SEED).standard_normal(w["n_hvf"])

    def batched():
        d = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=w["dtype"], ctx=ctx)
        B = sv.Batch.create(d, off, features=hvf, scale_max=SCALE_MAX)
        em = sv.batch_pca(B, w["npcs"], tol=1e-5, init=init, download=False)
        sv.batch_ann(B, em, w["k"], precision=w["knn"], download=False)
        ctx.sync()
        em.info["cells_per_block"] = B.cells_per_block
        return em

    def loop():
        out = []
        for c in per:
            d = sv.normalize_cells(c, scale_factor=SCALE_FACTOR, dtype=w["dtype"], ctx=ctx)
            S = sv.scale_features(d, scale_max=SCALE_MAX, features=hvf)
            em = sv.pca(S, w["npcs"], tol=1e-5, init=init, download=False)
            sv.ann(em, w["k"], precision=w["knn"], ctx=ctx, keep=True, download=False)
            out.append(em.stdev)
        ctx.sync()
        return out

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        ctx.sync()
        l0 = ctx.launches()
        t0 = time.perf_counter()
        r = None
        for _ in range(steps):
            r = fn()
        ctx.sync()
        return (time.perf_counter() - t0) / steps, (ctx.launches() - l0) / steps, r

    steps, warmup = max(1, min(args.steps, 3)), max(1, min(args.warmup, 2))
    clk = ClockSampler(0)
    clk.start()
    tb, lb, emb = timed(batched, steps, warmup)
    clocks = clk.stop()
    tl, ll, st_loop = timed(loop, 1, 1)
    sb = emb.stdev
    err = max(float(np.max(np.abs(sb[i] - st_loop[i]) / st_loop[i])) for i in range(w["n_samples"]))
    it = emb.info["iters"]
    out = {
        "metric": "cells/s, 64 samples (500-50,000 cells each) normalise→PCA30→kNN15: batched vs one sample per launch",
        "value": round(n / tb, 1), "unit": "cells/s", "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": round(tb * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic: seeded negative-binomial counts generated on the device (no dataset)",
        "config": {"workload": f"batched: {w['n_samples']} samples, {n} cells x {w['n_genes']} genes, "
                               f"{counts.nnz / n:.0f} nnz/cell, {w['n_hvf']} features, PCA {w['npcs']}, "
                               f"kNN {w['k']}",
                   "n_cells": n, "sample_cells_min": int(sizes.min()), "sample_cells_max": int(sizes.max()),
                   "nnz": counts.nnz, "depth_factor": round(D, 5), "value_dtype": w["dtype"],
                   "knn_kernel": w["knn"], "irlba_cycles_min": int(it.min()), "irlba_cycles_max": int(it.max()),
                   "xv_cells_per_block_autotuned": int(emb.info["cells_per_block"]),
                   "timing": "wall clock with the stream synchronised on both sides"},
        "loop": {"value": round(n / tl, 1), "ms_per_step": round(tl * 1e3, 3), "gpu_launches": int(ll)},
        "batched_vs_loop": round(tl / tb, 3),
        "stdev_rel_diff_batched_vs_loop_max": err,
        "gpu_launches": int(lb),
        "clocks": clocks,
    }
    if emit:
        print(json.dumps(out))
    return out


def _digit_table(vals, width):
    """Fixed-width digit rows of vals (ASCII) and the mask of their significant digits."""
    d = (vals[:, None] // (10 ** np.arange(width - 1, -1, -1, dtype=np.int64))[None, :]) % 10
    nz = np.logical_or.accumulate(d != 0, axis=1)
    nz[:, -1] = True
    return (d + 48).astype(np.uint8), nz


def mm_format(gene, cell, cnt, header, chunk=1 << 22):
    """MatrixMarket text of 1-based (gene, cell, count) triplets, built in host
    memory for the reader bench: digit rows are gathered from per-value tables
    (counts beyond the table are formatted directly), then the leading zeros
    are squeezed out chunk by chunk."""
    widths = (5, 7, 10)
    cols = [np.asarray(gene, np.int64), np.asarray(cell, np.int64), np.asarray(cnt, np.int64)]
    tabs = []
    for f, wd in zip(cols, widths):
        if len(f) and (f.min() < 0 or f.max() >= 10 ** wd):
            raise ValueError("field out of the formatter's range")
        top = int(min(f.max(initial=0), 1 << 20)) + 1
        tabs.append(_digit_table(np.arange(top, dtype=np.int64), wd))
    parts = [header.encode()]
    for a in range(0, len(cols[0]), chunk):
        m = min(chunk, len(cols[0]) - a)
        rows, keep = [], []
        for j, (f, wd) in enumerate(zip(cols, widths)):
            x = f[a:a + m]
            T, K = tabs[j]
            big = x >= len(T)
            xi = np.where(big, 0, x)
            r, k = T[xi], K[xi]
            if big.any():
                r[big], k[big] = _digit_table(x[big], wd)
            rows += [r, np.full((m, 1), ord("\n") if j == 2 else ord(" "), np.uint8)]
            keep += [k, np.ones((m, 1), bool)]
        parts.append(np.concatenate(rows, axis=1)[np.concatenate(keep, axis=1)].tobytes())
    return b"".join(parts)


def reader_bench(args, emit=True):
    """MatrixMarket reader (readMM as read_10X uses it): a 10X-layout text file
    (features x barcodes, entries ordered by cell) of seeded synthetic counts
    held in host memory, parsed into the device count matrix (both copies).
    Metric: text bytes per second, end to end through sv_counts_parse_mtx
    (the host-to-device copy of the text inside the timed region).  CPU
    baseline: the single-threaded C restatement of readMM + sparse + copy(X')
    on a bounded sample."""
    import __graft_entry__ as ge
    ge._build_module().build()
    sv = ge.load_package()
    ctx = sv.Context(0)
    w = dict(WORKLOADS["atlas"])
    n = args.cells or 50_000
    mu_g, s_c, cl, lfc = gen_params(w, n, SEED + 7)
    D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
    counts = sv.CountMatrix.generate(n, w["n_genes"], mu_g, s_c, cl, lfc, depth=D, dispersion=DISPERSION,
                                     seed=SEED + 7, ctx=ctx)
    R = counts.to_csr()
    del counts
    cell = np.repeat(np.arange(1, n + 1, dtype=np.int64), np.diff(R.indptr))
    t0 = time.perf_counter()
    text = mm_format(R.indices.astype(np.int64) + 1, cell, R.data,
                     f"%%MatrixMarket matrix coordinate integer general\n%\n{w['n_genes']} {n} {R.nnz}\n")
    gen_s = time.perf_counter() - t0
    steps, warmup = max(1, args.steps), max(3, args.warmup)
    for _ in range(warmup):
        X = sv.CountMatrix.parse_mtx(text, True, ctx=ctx)
        del X
    ctx.sync()
    clk = ClockSampler(0)
    clk.start()
    l0 = ctx.launches()
    t0 = time.perf_counter()
    for _ in range(steps):
        X = sv.CountMatrix.parse_mtx(text, True, ctx=ctx)
        del X
    ctx.sync()
    dt = (time.perf_counter() - t0) / steps
    clocks = clk.stop()
    launches = (ctx.launches() - l0) / steps
    ctx.profile_reset()
    ctx.profile(True)
    X = sv.CountMatrix.parse_mtx(text, True, ctx=ctx)
    ctx.sync()
    rep = ctx.profile_report()
    ctx.profile(False)
    ok = X.nnz == R.nnz and np.array_equal(X.to_csr().indptr, R.indptr)
    del X
    kern = {k: {"launches": c, "ms": round(ms, 3)} for k, (c, ms) in
            sorted(rep.items(), key=lambda kv: -kv[1][1])}
    parse_ms = rep.get("mtx_parse", (1, float("nan")))[1]
    nbytes = len(text)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    # mtx_parse reads every text byte and 8 bytes of line end per entry, and
    # writes 12 bytes per entry (cell, gene, count)
    parse_bytes = nbytes + 20 * R.nnz
    cpu = None
    if not args.no_cpu:
        from oracle import mtx as mo
        ns = min(n, 4000)
        hdr = f"%%MatrixMarket matrix coordinate integer general\n{w['n_genes']} {ns} {int(R.indptr[ns])}\n"
        k = int(R.indptr[ns])
        sample = mm_format(R.indices[:k].astype(np.int64) + 1, cell[:k], R.data[:k], hdr)
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 10.0 or reps == 0:
            mo.parse(sample, True)
            reps += 1
        cs = (time.perf_counter() - t0) / reps
        cpu = {"value": round(len(sample) / cs / 1e6, 2), "unit": "MB/s", "cores": 1, "kind": "port",
               "sample": f"{ns} cells ({len(sample) / 1e6:.1f} MB) of the same file, C restatement of "
                         f"readMM + sparse + copy(X'), single thread"}
    out = {
        "metric": "MatrixMarket text → device count matrix (CSC + CSR), bytes/s",
        "value": round(nbytes / dt / 1e6, 1), "unit": "MB/s", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic: seeded negative-binomial counts written as 10X-layout MatrixMarket text",
        "config": {"workload": f"reader: {n} cells x {w['n_genes']} genes, {R.nnz} entries, "
                               f"{nbytes / 1e9:.2f} GB of text in host memory",
                   "entries": int(R.nnz), "text_bytes": nbytes,
                   "l2": "text larger than L2 (129 MB)",
                   "timing": "wall clock with the stream synchronised on both sides"},
        "e2e": {"value": round(nbytes / dt / 1e6, 1), "unit": "MB/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": 0},
        "entries_per_s": round(R.nnz / dt, 1),
        "parse_kernel": {"bytes": parse_bytes, "ms": round(parse_ms, 3),
                         "gbs": round(parse_bytes / (parse_ms / 1e3) / 1e9, 1),
                         "frac_of_hbm": round(parse_bytes / (parse_ms / 1e3) / 1e9 / hbm, 3)},
        "kernels_ms": kern,
        "device_matches_source": bool(ok),
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "generate_s": round(gen_s, 2),
    }
    if emit:
        print(json.dumps(out))
    return out


def extras(args):
    """The batched-samples and reader measurements as compact fields of the
    default line (after its timed region), each guarded: a failure is recorded,
    not raised."""
    import argparse as _ap
    res = {}
    sub = _ap.Namespace(**vars(args))
    sub.cells = 0
    sub.steps, sub.warmup = 2, 1
    try:
        b = batched_bench(sub, emit=False)
        res["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "loop", "batched_vs_loop",
                                             "stdev_rel_diff_batched_vs_loop_max", "gpu_launches")}
        res["batched"]["workload"] = b["config"]["workload"]
    except Exception as e:   # recorded in the line, the main measurement stands
        res["batched"] = {"error": repr(e)[:300]}
    sub.steps, sub.warmup = 3, 3
    try:
        r = reader_bench(sub, emit=False)
        res["reader"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "entries_per_s", "parse_kernel",
                                            "device_matches_source", "cpu_baseline", "gpu_launches")}
        res["reader"]["workload"] = r["config"]["workload"]
    except Exception as e:
        res["reader"] = {"error": repr(e)[:300]}
    return res


def kernel_case(args):
    """Small inputs that still exceed L2, for kernel-level profiler captures
    (a few GB on the device):
      irlba: a random sparse 600,000 x 3,000 CenteredMatrix (40 non-zeros per
             cell, FP32) and 3 restart cycles of irlba 50 -- the Lanczos kernels
             on a 274 MB cell-side basis;
      knn:   400,000 x 50 mixture points, k = 20, BF16 tensor-core path;
      prep:  filter_counts and find_variable_features(:vst) on 200,000 atlas
             cells generated on the device."""
    import __graft_entry__ as ge
    import scipy.sparse as sp
    ge._build_module().build()
    sv = ge.load_package()
    ctx = sv.Context(0)
    rng = np.random.default_rng(SEED)
    if args.kernel_case == "irlba":
        n, nf, per = args.cells or 600_000, 3000, 40
        cols = rng.integers(0, nf, n * per)
        rows = np.repeat(np.arange(n), per)
        X = sp.csc_matrix((rng.random(n * per).astype(np.float32) * 4, (rows, cols)), shape=(n, nf))
        X.sum_duplicates()
        mu = np.asarray(X.mean(axis=0)).ravel()
        S = sv.CenteredMatrix.from_sparse(X, mu, dtype="float32", ctx=ctx)
        t0 = time.perf_counter()
        try:
            sv.irlba(S, 50, tol=1e-5, maxit=3)
        except sv.ConvergenceError:
            pass
        ctx.sync()
        out = {"kernel_case": "irlba", "n_cells": n, "features": nf, "nnz": int(X.nnz),
               "cycles": 3, "s": round(time.perf_counter() - t0, 4)}
    elif args.kernel_case == "prep":
        # the steps before the path: filter_counts and find_variable_features(:vst)
        w = dict(WORKLOADS["atlas"])
        n = args.cells or 200_000
        mu_g, s_c, cl, lfc = gen_params(w, n, SEED)
        D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
        counts = sv.CountMatrix.generate(n, w["n_genes"], mu_g, s_c, cl, lfc, depth=D,
                                         dispersion=DISPERSION, seed=SEED, ctx=ctx)
        t0 = time.perf_counter()
        F, ci, fi = sv.filter_counts(counts, min_cells=3, min_features=200)
        t1 = time.perf_counter()
        feats, _ = sv.find_variable_features(F, w["n_hvf"])
        ctx.sync()
        out = {"kernel_case": "prep", "n_cells": n, "kept_cells": int(ci.sum()), "kept_genes": int(fi.sum()),
               "filter_s": round(t1 - t0, 4), "vst_s": round(time.perf_counter() - t1, 4)}
        # per-kernel device times (CUDA events) of vst under each loess surface
        sel = {}
        for surf in ("interpolate", "hermite", "direct"):
            ctx.profile(True)
            ctx.profile_reset()
            t2 = time.perf_counter()
            f2, _ = sv.find_variable_features(F, w["n_hvf"], loess_surface=surf)
            ctx.sync()
            out[f"vst_{surf}"] = {"s": round(time.perf_counter() - t2, 4),
                                  "kernels_ms": {k: round(v[1], 3) for k, v in ctx.profile_report().items()}}
            ctx.profile(False)
            sel[surf] = set(f2.tolist())
        out["vst_selection_overlap_vs_direct"] = {
            s: round(len(sel[s] & sel["direct"]) / max(1, len(sel["direct"])), 4) for s in ("interpolate", "hermite")}
    else:
        n, d = args.cells or 400_000, 50
        means = rng.normal(0, 4, (60, d))
        X = means[rng.integers(0, 60, n)] + rng.standard_normal((n, d))
        X = (X / np.sqrt(np.arange(1, d + 1))).astype(np.float32)
        t0 = time.perf_counter()
        sv.ann(X, 20, precision="bf16" if knn_tc_available(sv, ctx) else "fp32", ctx=ctx)
        out = {"kernel_case": "knn", "n": n, "d": d, "k": 20, "s": round(time.perf_counter() - t0, 4)}
    print(json.dumps(out))


def principal_angles(A, B):
    """Principal angles (radians) between the column spaces of A and B."""
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    c = np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0)
    return np.arccos(c)


def exact_knn_sample(Z, q, k, include_self=True, block=262144):
    """Exact FP64 Euclidean neighbours of the query rows q against all of Z
    (0-based, the query itself included): the recall reference."""
    Z = np.asarray(Z, dtype=np.float64)
    Q = Z[q]
    sqq = np.einsum("ij,ij->i", Q, Q)
    ci, cd = [], []
    for s0 in range(0, Z.shape[0], block):
        B = Z[s0:s0 + block]
        D = sqq[:, None] + np.einsum("ij,ij->i", B, B)[None, :] - 2.0 * (Q @ B.T)
        inb = (q >= s0) & (q < s0 + len(B))
        D[np.nonzero(inb)[0], q[inb] - s0] = -1.0
        m = min(k, len(B))
        part = np.argpartition(D, m - 1, axis=1)[:, :m]
        ci.append(part + s0)
        cd.append(np.take_along_axis(D, part, axis=1))
    ci = np.concatenate(ci, axis=1)
    cd = np.concatenate(cd, axis=1)
    order = np.argsort(cd, axis=1, kind="stable")[:, :k]
    return np.take_along_axis(ci, order, axis=1)


def knn_stress(sv, ctx, with_fp32):
    """kNN stress case: 2,000,000 x 50 FP32 points of a 60-component Gaussian
    mixture (means ~ N(0, 4^2), dimension i scaled by 1/sqrt(i)), k = 30: BF16
    tensor-core candidates (64 per point) + FP32 re-rank through the host API,
    recall@30 against FP64 brute force on 500 sampled points."""
    n, d, k = 2_000_000, 50, 30
    rng = np.random.default_rng(SEED + 5)
    means = rng.normal(0, 4, (60, d))
    X = means[rng.integers(0, 60, n)]
    X += rng.standard_normal((n, d))
    X *= 1.0 / np.sqrt(np.arange(1, d + 1))
    X = X.astype(np.float32)
    sv.ann(X[:4096], k, precision="bf16", ctx=ctx)          # warm-up
    t0 = time.perf_counter()
    idx, _ = sv.ann(X, k, precision="bf16", ctx=ctx)
    t_bf16 = time.perf_counter() - t0
    q = np.random.default_rng(11).choice(n, 500, replace=False)
    ref = exact_knn_sample(X, q, k)
    hits = sum(len(set(a - 1) & set(b)) for a, b in zip(idx[q], ref))
    flops = 2.0 * n * n * d
    out = {"n": n, "d": d, "k": k, "bf16_s": round(t_bf16, 4),
           "bf16_distance_tflops": round(flops / t_bf16 / 1e12, 1),
           "recall_at_30": hits / ref.size, "recall_queries": 500,
           "note": "host API: includes the 400 MB upload and the result download"}
    if with_fp32:
        t0 = time.perf_counter()
        sv.ann(X, k, precision="fp32", ctx=ctx)
        t32 = time.perf_counter() - t0
        out["fp32_cuda_core_s"] = round(t32, 4)
        out["bf16_speedup_vs_fp32"] = round(t32 / t_bf16, 2)
    return out


# a PC counts as well separated when its singular value lies at least this far
# (relative to sigma_1) from both neighbours: with irlba's tol = 1e-5 its
# Ritz residual is at most 1e-5 sigma_1, so its angle is at most ~1e-2 rad by
# the residual bound and in practice far below 1e-4
SEP_GAP = 1e-3


def _pca_form(sv, ctx, counts, hvf, dtype, npcs, tol, init):
    d = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=dtype, ctx=ctx)
    S = sv.scale_features(d, scale_max=SCALE_MAX, features=hvf)
    em = sv.pca(S, npcs, tol=tol, init=init, download=True)
    del d, S
    return em


def pc_errors(em, s_ref, V_ref, npcs):
    """Errors of one embedding against the FP64 reference (npcs + 1 singular
    values, so that the gap below the last PC is known): singular values, the
    angle of each PC, the largest angle over the well-separated PCs, and the
    angle of the largest leading block that ends at a wide gap."""
    s = em.stdev
    sr = s_ref[:npcs + 1]
    d_next = (sr[:npcs] - sr[1:npcs + 1]) / sr[0]
    d_prev = np.r_[np.inf, d_next[:-1]]
    sep = np.minimum(d_prev, d_next) >= SEP_GAP
    per = np.arccos(np.clip(np.abs(np.einsum("ij,ij->j", em.basis, V_ref[:, :npcs])), 0.0, 1.0))
    wide = np.nonzero(d_next >= SEP_GAP)[0]
    kb = int(wide[-1]) + 1 if len(wide) else 0
    out = {"sigma_rel_err_max": float(np.max(np.abs(s - sr[:npcs]) / sr[:npcs])),
           "pc_angle_max_rad": float(per.max()),
           "pc_angle_max_separated_rad": float(per[sep].max()) if sep.any() else None,
           "separated_pcs": int(sep.sum()),
           "leading_block": {"k": kb, "gap_rel": float(d_next[kb - 1]) if kb else None,
                             "angle_rad": float(principal_angles(em.basis[:, :kb],
                                                                 V_ref[:, :kb]).max()) if kb else None},
           "subspace_angle_all_rad": float(principal_angles(em.basis, V_ref[:, :npcs]).max()),
           "pc_angles_rad": [float(f"{x:.2g}") for x in per]}
    return out, d_next, d_prev


def accuracy(sv, ctx, counts, hvf, w, init, form, n_queries=1000):
    """Errors of the measured form (and of the plain FP32 form) against the same
    pipeline in FP64 at tol 1e-8: relative error of the singular values, the
    angle of every PC next to its gap, the largest angle over the well-separated
    PCs, the leading block's subspace angle, and kNN recall@k against exact FP64
    neighbours (brute force on the host, for a sample of query cells, over the
    measured form's coordinates)."""
    npcs = w["npcs"]
    em64 = _pca_form(sv, ctx, counts, hvf, "float64", npcs + 1, 1e-8, init)
    s64, V64 = em64.stdev, em64.basis
    em = _pca_form(sv, ctx, counts, hvf, form[0], npcs, 1e-5, init)
    out, d_next, d_prev = pc_errors(em, s64, V64, npcs)
    out["pc_gaps_rel"] = [float(f"{x:.2g}") for x in np.minimum(d_prev, d_next)]
    out["sigma_gap_last"] = float(s64[npcs - 1] / s64[npcs] - 1)      # sigma_50 / sigma_51 - 1
    out["separation_threshold"] = SEP_GAP
    if form[0] != "float32":
        em32 = _pca_form(sv, ctx, counts, hvf, "float32", npcs, 1e-5, init)
        e32, _, _ = pc_errors(em32, s64, V64, npcs)
        out["plain_fp32"] = e32
        del em32
    if form[0] == "bfloat16":
        out["bf16_cause"] = ("storage: BF16 rounding of the normalised values (unit roundoff 2^-9) "
                             "perturbs the matrix itself; the same angles appear at tol 1e-8, while "
                             "FP32 / FP64 values at tol 1e-5 stay below 1e-5 rad on separated PCs")
    idx, _ = sv.ann(em, w["k"], precision=form[1], ctx=ctx)
    Z = np.ascontiguousarray(em.coordinates)
    n = Z.shape[0]
    q = np.random.default_rng(7).choice(n, min(n_queries, n), replace=False)
    sq = np.einsum("ij,ij->i", Z, Z)
    hits = 0
    for b in range(0, len(q), 250):
        qq = q[b:b + 250]
        D = sq[qq, None] + sq[None, :] - 2.0 * (Z[qq] @ Z.T)
        D[np.arange(len(qq)), qq] = -1.0
        part = np.argpartition(D, w["k"] - 1, axis=1)[:, :w["k"]]
        for r, i in enumerate(qq):
            hits += len(set(part[r]) & set(idx[i] - 1))
    out["knn_recall"] = hits / (len(q) * w["k"])
    out["knn_recall_queries"] = int(len(q))
    out["reference"] = ("same pipeline in FP64 on the device (normalised values FP64, FP64 products), "
                        f"irlba tol 1e-8, {npcs + 1} singular values")
    return out


def accuracy_study(args):
    """Separates the causes of the PC errors at the atlas size: every value
    storage type (BF16, FP32, FP64) at irlba tol 1e-5 (the reference default)
    and 1e-8, against FP64 values at tol 1e-10 with npcs + 7 singular values."""
    import __graft_entry__ as ge
    ge._build_module().build()
    sv = ge.load_package()
    ctx = sv.Context(0)
    w = dict(WORKLOADS[args.workload])
    if args.cells:
        w["n_cells"] = args.cells
    n, npcs = w["n_cells"], w["npcs"]
    mu_g, s_c, cl, lfc = gen_params(w, n, SEED)
    D = calibrate_depth(mu_g, s_c, cl, lfc, w["nnz_per_cell"])
    counts = sv.CountMatrix.generate(n, w["n_genes"], mu_g, s_c, cl, lfc, depth=D,
                                     dispersion=DISPERSION, seed=SEED, ctx=ctx)
    d0 = sv.normalize_cells(counts, scale_factor=SCALE_FACTOR, dtype=w["dtype"], ctx=ctx)
    _, var = d0.gene_moments()
    hvf = np.sort(np.argsort(-var, kind="stable")[: w["n_hvf"]]) + 1
    del d0
    init = np.random.default_rng(SEED).standard_normal(w["n_hvf"])
    ref = _pca_form(sv, ctx, counts, hvf, "float64", npcs + 7, 1e-10, init)
    out = {"workload": args.workload, "n_cells": n, "reference": f"float64 values, tol 1e-10, {npcs + 7} values",
           "sigma_ref": [round(float(x), 4) for x in ref.stdev]}
    for dtype in ("bfloat16", "float32", "float64"):
        for tol in (1e-5, 1e-8):
            t0 = time.perf_counter()
            em = _pca_form(sv, ctx, counts, hvf, dtype, npcs, tol, init)
            e, d_next, d_prev = pc_errors(em, ref.stdev, ref.basis, npcs)
            e["pca_s"] = round(time.perf_counter() - t0, 2)
            out[f"{dtype}_tol{tol:g}"] = e
    out["pc_gaps_rel"] = [float(f"{x:.2g}") for x in np.minimum(d_prev, d_next)]
    print(json.dumps(out))


def knn_tc_available(sv, ctx):
    try:
        X = np.random.default_rng(0).standard_normal((256, 16))
        sv.ann(X, 4, precision="bf16", ctx=ctx)
        return True
    except sv.SeveroGPUError:
        return False


def reference_arm(args, w, td, rank, world):
    """The reference's CPU path, restated in C/OpenMP (the Julia package and
    its binary dependency cannot run here), on the host cores; its kNN is an
    approximate search of the reference's kind (random-projection trees).  Warm-up steps
    run a 2,000-cell sample; the first timed step a 130,000-cell sample (a
    tenth of the atlas), the others a 32,500-cell sample, all prefixes of one
    generated sample.  Each stage is extrapolated to the atlas from the large
    sample by its growth measured between the two sizes.  Rank 0 alone works
    under torchrun."""
    if rank != 0:
        if td is not None:
            td.destroy_process_group()
        return
    from oracle import cpu_path
    n = w["n_cells"]
    big, small = min(REF_LARGE, n), min(REF_SMALL, n)
    sizes = [min(REF_WARM, n)] * args.warmup + [big] + [small] * max(1, args.steps - 1)
    params = cpu_params(w, big)
    nt = cpu_path.threads()
    t_all = time.perf_counter()
    recs = cpu_path.run_in_subprocess(params, sizes, nt, seed=SEED, n_hvf=w["n_hvf"], npcs=w["npcs"],
                                      k=w["k"])
    wall = time.perf_counter() - t_all
    timed = recs[args.warmup:]
    value, st_full, alpha = cpu_model(timed, n)
    measured_s = sum(sum(r["stages_s"].values()) for r in timed)
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * n / value, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded negative-binomial counts (C generator), bounded samples per step",
        "config": {"workload": f"{args.workload}: {n} cells x {w['n_genes']} genes",
                   "n_cells": n, "sample_cells": {"large": big, "small": small, "warmup": min(REF_WARM, n)}},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": "cells/s", "cores": nt, "kind": "port",
                         "sample": (f"C/OpenMP restatement of the reference path (FP64) on {nt} host "
                                    f"threads: step 1 on {big} cells, steps 2..{args.steps} on {small} "
                                    f"cells; each stage extrapolated to {n} cells by its growth "
                                    f"measured between the two sizes (exponents {alpha}); kNN by "
                                    f"random-projection trees (ntables = 2 d, the reference's default) "
                                    f"+ one neighbour-of-neighbour round, recall@{w['k']} "
                                    f"{timed[0].get('knn_recall')} against exact search on 500 cells; "
                                    f"measured region {measured_s:.1f} s, wall {wall:.1f} s")},
        "stages_s_at_full": {k_: round(v, 2) for k_, v in st_full.items()},
        "measured_large": {k_: round(v, 3) for k_, v in timed[0]["stages_s"].items()},
        "knn_recall_large": timed[0].get("knn_recall"),
        "fits_in_driver_run": bool(wall < 900),
        "e2e": {"value": round(value, 3), "unit": "cells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    if td is not None:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
