#!/usr/bin/env python
"""Benchmark of the Fast-Higashi fit hot path on one GB300: cells/s for RWR + 30 ALS iterations.

A step is one fit of the workload (default c3: 10,000 cells, 22 autosomes at 500 kb, R=64,
band 30): the contact build, the partial RWR of every tile and 30 iterations of the
PARAFAC2-like ALS (per-bin polar, SVD_term, meta polar, projections, CP-ALS), from a fixed
initial state (init_params runs once, untimed, as the metric states).

  value       the tensor-core form (precision="bf16x2": tcgen05 RWR and X passes, X as two
              bf16 planes), device-timed with CUDA events, contacts resident in HBM
  plain_fp32  the plain fp32 drop-in on the same GPU and state, timed the same way, with
              the speed-up of the headline form over it
  e2e         the public API (Fast_Higashi_core.fit on host Sparse data) with the COO H2D and
              the embedding / loss D2H inside the timed region
  input_packing / post_processing  the rows either side of the fit, each device-timed on
              its own: fh_pack_chromosome over every chromosome from raw contacts in HBM, and
              fetch_cell_embedding + correct_batch_linear for every cell (--no-extras skips)
  --impl reference   the reference's own Fast_Higashi_core (installed under baseline/_ref) on
                     the host CPU, all cores, one ALS iteration per step on a cell sample,
                     extrapolated to the workload's cells and iterations (cpu_baseline says how)
  --hbm-budget-gb G  both forms held within G GB of device memory (X's last chromosomes
                     streamed from page-locked host memory, contacts built one dataset at a
                     time): the 50,000-cell, R = 128 case is --config c5 --hbm-budget-gb 180;
                     its own JSON line with the memory, the X plan and the host-link bytes

Multi-GPU runs (torchrun) are independent replicas: the fit does not shard (scaling weak).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "fast-higashi_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "cells/sec for RWR + ALS fit, BF16-batched vs plain FP32 on GB300 at stated error"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default=None,
                    help="workload: c1..c5 (default c3, 10,000 cells at 500 kb, the one the "
                         "BF16-batched vs plain FP32 target is set on; c4 with --grad)")
    ap.add_argument("--grad", action="store_true",
                    help="time the differentiable reconstruction loss (forward + backward) "
                         "instead of the fit; prints its own JSON line")
    ap.add_argument("--iters", type=int, default=None, help="ALS iterations (default: the workload's 30)")
    ap.add_argument("--cells", type=int, default=None,
                    help="run the workload's shapes with this many cells instead (a reduced "
                         "case, named as such in config.workload; never the headline)")
    ap.add_argument("--sample-cells", type=int, default=128,
                    help="cells of the reference's CPU sample (at least the rank R)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own torch path on the GPU (context)")
    ap.add_argument("--gpu-sample-cells", type=int, default=2000,
                    help="cells of the reference's GPU sample")
    ap.add_argument("--precision", default="bf16x2", choices=["fp32", "bf16x2", "bf16"],
                    help="form timed for the headline: bf16x2 (default) the tensor-core form, X "
                         "as two bf16 planes; bf16 one plane; fp32 the plain drop-in")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip timing the plain fp32 form beside the headline form")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the input-packing and post-processing measurements")
    ap.add_argument("--extras-only", action="store_true",
                    help="only the input-packing and post-processing measurements (after the "
                         "GPU init_params), one JSON line")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the FP64 fit that states both forms' embedding error")
    ap.add_argument("--hbm-budget-gb", type=float, default=None,
                    help="hold each fit within this many GB of device memory: X's last "
                         "chromosomes stream from host memory when X does not fit, the contact "
                         "segments are built one dataset at a time (the 50,000-cell c5 case: "
                         "--config c5 --hbm-budget-gb 180); prints its own JSON line")
    args = ap.parse_args()
    args.config = args.config or ("c4" if args.grad else "c3")
    return args


def dist_setup():
    """One process per GPU under torchrun (NCCL); gloo where no GPU is visible (the host-side
    logic of the N > 1 runs, exercised by the CPU tests)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 0, 1
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist.init_process_group("gloo")
    return rank, local, ws


def max_over_ranks(x, ws):
    """The largest of every rank's x (a one-element tensor): whole-job time is the slowest
    replica's."""
    if ws > 1:
        import torch.distributed as dist
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return x


def make_workload(name, seed=0, cells=None):
    import dataclasses
    from fh_gb300 import synth
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    w = synth.workload(name)
    if cells:
        w = dataclasses.replace(w, n_cells=int(cells), name="%s at %d cells" % (name, cells))
    coo, _ = synth.generate(w, seed=seed)
    ds = []
    for (idx, val, shape), cname, nb in zip(coo, w.chrom_names, w.chrom_bins):
        bsb, bsc = synth.recommend_batches(w, nb, w.n_cells)
        ds.append(Chrom_Dataset(Sparse(idx, val, shape, copy=False), bsb, bsc, compact=True,
                                flank=w.band, chrom=cname, resolution=w.resolution))
    # the contacts in page-locked host memory, as the reference's datasets pin theirs
    # (Chrom_Dataset.pin_memory): every step's host-to-device copy reads pinned memory
    for d in ds:
        d.pin_memory()
    return w, coo, ds


class _Null:
    def __enter__(self):
        return None

    def __exit__(self, *a):
        return False


def aligned_diff(E, Eref):
    """Relative Frobenius difference of E after the orthogonal Procrustes rotation onto Eref
    (two fits' embeddings agree up to a rotation)."""
    import torch
    E, Eref = E.double(), Eref.double()
    U, _, Vh = torch.linalg.svd(E.T @ Eref)
    return float(torch.linalg.norm(E @ (U @ Vh) - Eref) / torch.linalg.norm(Eref))


class Clocks:
    """nvidia-smi samples (200 ms) of the SM clock and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.lines, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM traffic per launch / algorithmic X bytes of the tensor-core X passes, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the fit's passes at 2,000 cells x 301,461
# band rows; the bench scales it by the X bytes of its own workload (cells x band rows).
XPASS_TRAFFIC_RATIO = {"xe": (2.447e9 + 74.7e6) / 2.412e9, "xg": (2.497e9 + 8.7e6) / 2.412e9}


def autotune_summary():
    """The schedules the autotuner timed in this process: {knob and shape: candidate -> ms,
    choice}."""
    from fh_gb300 import autotune
    return {k.split("|", 1)[1]: {"ms": {str(c): round(t, 4) for c, t in times.items()},
                                  "choice": best}
            for k, times, best in autotune.default_tuner().log}


# DRAM bytes per launch of the per-bin polar kernel per bin row, from its ncu capture at 2,000
# cells (78.8 MB read + 94.6 MB written over 2,887 bin rows: W rows in, U and G^T out); the
# bench scales it by its own bin rows.
PROCRUSTES_TRAFFIC_PER_ROW = (78.77e6 + 94.60e6) / 2887


def family_work(eng, iters_sched=None):
    """Algorithmic work per launch of each kernel family of the fit, as (amount, unit, bound):
      rwr         sum over tiles of cells x 2 b^2 n (1 + epochs): the transition matrix's
                  A A^T and one b x b by b x n product per walk epoch (the tensor-core form runs
                  each product as three split-bf16 products; only one is counted)
      xe, xg      the X bytes one pass reads: cells x band rows x bytes per element
      procrustes  per bin row (n columns, rank r, meta rank R): temp 2nRr + Householder QR
                  2nr^2 - 2r^3/3 + the polar factor of the r x r triangle counted as ten r x r
                  products (20 r^3, the class of its Newton and Newton-Schulz steps) + forming U
                  4nr^2 - 2r^3 + G^T 2nrR, fp32
      meta_polar  cells x R^2 (fp64 Gram, one triangle) + 2 cells x R^2 (apply)
      project_y   bytes of U, W read and Y written
      cp_als      per sweep and bin row 6 r^2 R (three MTTKRPs), times the mean sweeps per call
    """
    t = eng.tiles
    b = t["rows"].astype(np.float64)
    n = t["width"].astype(np.float64)
    r = t["rank"].astype(np.float64)
    ep = t["n_rwr"].astype(np.float64)
    R, rp, ld = float(eng.R), eng.rp, eng.ld
    xel = 2 * eng.planes if eng.bf16 else 4
    nr = np.repeat(n, t["rows"])
    rr = np.repeat(r, t["rows"])
    proc = float((2 * nr * R * rr + 2 * nr * rr ** 2 - 2 * rr ** 3 / 3 + 20 * rr ** 3 +
                  4 * nr * rr ** 2 - 2 * rr ** 3 + 2 * nr * rr * R).sum())
    sweeps = float(np.mean(iters_sched)) if iters_sched else 1.0
    return {
        "rwr": (eng.Ct * float((2 * b * b * n * (1 + ep)).sum()), "FLOP",
                "tensor" if eng.bf16 else "fp32"),
        "xe": (float(eng.C) * eng.rows * xel, "B", "hbm"),
        "xg": (float(eng.C) * eng.rows * xel, "B", "hbm"),
        "procrustes": (proc, "FLOP", "fp32"),
        "meta_polar": (3.0 * eng.C * R * R, "FLOP", "fp64"),
        "project_y": (4.0 * (eng.u_size + eng.rows * rp + eng.nb * ld * rp), "B", "hbm"),
        "cp_als": (sweeps * float((6 * rr ** 2 * R).sum()), "FLOP", "fp32"),
    }


def family_rooflines(eng, kt, sm_max_mhz, sched):
    """Per kernel family: algorithmic work per launch, its CUDA-event time (mean over the
    launches of one instrumented fit), the rate, the bound and its fraction of that bound's
    peak.  Peaks: HBM and bf16 tensor from MEASURED_PEAKS.json (the sustained bf16 figure: these
    kernels run inside a long step); fp32 and fp64 CUDA-core rates are nominal at the sampled
    maximum SM clock (128 fp32 and 2 fp64 FMA per SM per clock, 152 SMs)."""
    hbm, _, peak_kind = peaks()
    bf16s = sustained_bf16()
    mhz = sm_max_mhz or 2070.0
    fp32 = 2 * 128 * 152 * mhz * 1e6 / 1e12
    peak = {"hbm": (hbm, "GB/s", peak_kind), "tensor": (bf16s, "TFLOP/s", peak_kind),
            "fp32": (fp32, "TFLOP/s", "nominal"), "fp64": (fp32 / 64, "TFLOP/s", "nominal")}
    out = []
    for fam, (work, unit, bound) in family_work(eng, sched).items():
        if fam not in kt:
            continue
        sec = kt[fam]["mean_ms"] / 1000.0
        rate = work / sec / (1e9 if unit == "B" else 1e12)
        pk, pu, pkind = peak[bound]
        out.append({"kernel": fam, "bound": bound, "achieved": rate, "peak": pk, "unit": pu,
                    "frac": rate / pk, "peak_kind": pkind, "work_per_launch": work,
                    "work_unit": unit, "ms_per_launch": kt[fam]["mean_ms"],
                    "launches_per_fit": kt[fam]["calls"]})
    return out


def sustained_bf16():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops_sustained"])
    except (OSError, KeyError, ValueError):
        return 1700.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback"


# --------------------------------------------------------------------------------------
REF_DIR = os.path.join(ROOT, "baseline", "_ref")


def import_reference(path=REF_DIR):
    """The reference package (fasthigashi) from its pip --target install, unmodified.

    Third-party modules its fit path imports are used where installed.  Where the host lacks
    one, a stand-in is placed in sys.modules for the import only (the reference binds the
    names it needs at import time) and named in the returned notes:
      pandas      util.py:2, parafac_integrative.py:5; nothing on the fit path uses it: an
                  empty module
      sklearn     TruncatedSVD (init_params, parafac2_intergrative.py:257) and NearestNeighbors
                  (util.py:7, unused): TruncatedSVD.fit_transform as numpy's SVD of the same
                  matrix (init is not timed); NearestNeighbors raises if called
      opt_einsum  contract (parafac2_intergrative.py:374,422,522,629; parafac_integrative.py:
                  57,82): torch.einsum of the same subscripts
    Returns (modules, notes)."""
    import importlib.util
    import types
    notes = []
    stubs = {}
    if importlib.util.find_spec("pandas") is None:
        stubs["pandas"] = types.ModuleType("pandas")
        notes.append("pandas: empty module (no use on the fit path)")
    if importlib.util.find_spec("sklearn") is None:
        sk, dec, nei = (types.ModuleType(n) for n in ("sklearn", "sklearn.decomposition",
                                                       "sklearn.neighbors"))

        class TruncatedSVD:
            def __init__(self, n_components=2, **kw):
                self.k = int(n_components)

            def fit_transform(self, X):
                U, S, _ = np.linalg.svd(np.asarray(X, dtype=np.float64), full_matrices=False)
                return U[:, :self.k] * S[:self.k]

        class NearestNeighbors:
            def __init__(self, *a, **kw):
                raise RuntimeError("NearestNeighbors is not available on this host")

        dec.TruncatedSVD = TruncatedSVD
        nei.NearestNeighbors = NearestNeighbors
        sk.decomposition, sk.neighbors = dec, nei
        stubs.update({"sklearn": sk, "sklearn.decomposition": dec, "sklearn.neighbors": nei})
        notes.append("sklearn: TruncatedSVD as numpy SVD (init only, untimed)")
    if importlib.util.find_spec("opt_einsum") is None:
        import torch
        oe = types.ModuleType("opt_einsum")
        oe.contract = lambda eq, *ops, **kw: torch.einsum(eq, *ops)
        stubs["opt_einsum"] = oe
        notes.append("opt_einsum: contract as torch.einsum")
    if not os.path.isdir(os.path.join(path, "fasthigashi")):
        raise FileNotFoundError("the reference is not installed under %s" % path)
    if path not in sys.path:
        sys.path.insert(0, path)
    added = [k for k in stubs if k not in sys.modules]
    for k in added:
        sys.modules[k] = stubs[k]
    try:
        import fasthigashi.parafac2_intergrative as core
        import fasthigashi.sparse_for_schic as sfs
    finally:
        for k in added:
            del sys.modules[k]
    return {"core": core, "sparse": sfs}, notes


def reference_datasets(ref, w, coo):
    """The reference's own Sparse / Chrom_Dataset objects for a workload's COO, with the
    batching the GPU arm uses (one cell batch; bin batches per FastHigashi_Wrapper.py:501,
    507-512).  Sparse is built with copy=True: its np.array(shape, copy=False) rejects the
    shape tuple under NumPy 2 (same values)."""
    from fh_gb300 import synth
    sfs = ref["sparse"]
    out = []
    for (idx, val, shape), name, nb in zip(coo, w.chrom_names, w.chrom_bins):
        bsb, _ = synth.recommend_batches(w, nb, w.n_cells)
        obj = sfs.Sparse(idx.copy(), val.copy(), shape, copy=True)
        obj.sort_indices()
        out.append(sfs.Chrom_Dataset(tensor=obj, bs_bin=bsb, bs_cell=w.n_cells, good_qc_num=-1,
                                     kind="hic", upper_sim=False, compact=True, flank=w.band,
                                     chrom=name, resolution=w.resolution))
    return out


class _Quiet:
    """Silences the reference's progress printing and bars (stdout, stderr) while it runs."""

    def __enter__(self):
        self.saved = (sys.stdout, sys.stderr)
        sys.stdout = sys.stderr = open(os.devnull, "w")

    def __exit__(self, *a):
        sys.stdout.close()
        sys.stdout, sys.stderr = self.saved
        return False


def reference_fit_rate(config, n_cells, iters, steps, warmup, device="cpu"):
    """Times the reference's own Fast_Higashi_core.fit on the host CPU (all cores), or on
    device="cuda" its torch path on this GPU, on a cell sample of the workload: the
    reference's init_params once (untimed), then warmup + steps fits of one ALS iteration each
    from that state (every iteration recomputes the RWR of each tile, as the reference does).
    One more fit at half the sample separates the cost that does not grow with cells (the
    per-bin polar factors, CP-ALS); the full fit of the workload's cells is extrapolated as
    iters x (fixed + per-cell x cells).  Returns (cells/s, step seconds, description dict)."""
    import dataclasses
    import torch
    from fh_gb300 import synth
    ref, notes = import_reference()
    core = ref["core"]
    threads = os.cpu_count()
    torch.set_num_threads(threads)
    w_full = synth.workload(config)
    cpu = torch.device(device)
    on_gpu = cpu.type == "cuda"

    def sample(c):
        w = dataclasses.replace(w_full, n_cells=int(c))
        coo, _ = synth.generate(w, seed=0)
        return w, reference_datasets(ref, w, coo)

    def one_fit(w, ds, state):
        m = core.Fast_Higashi_core(rank=w.rank, off_diag=w.band, res_list=[w.resolution]).to(cpu)
        if state is None:
            np.random.seed(0)
            torch.manual_seed(0)
            with _Quiet():
                m.fit(ds, size_ratio=w.dim1, n_iter_max=0, n_iter_parafac=1, do_conv=False,
                      do_rwr=True, do_col=False, tol=0, run_init=True)
            return m, None
        m.A_list = [a.clone() for a in state[0]]
        m.B_dict = {k: v.clone() for k, v in state[1].items()}
        m.D_dict = {k: v.clone() for k, v in state[2].items()}
        m.meta_embedding = state[3].clone()
        m.n_i = state[4].copy()
        m.bin_cov_list = [b.clone() if torch.is_tensor(b) else b for b in state[5]]
        m.bad_bin_cov_list = list(state[6])
        if on_gpu:
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        with _Quiet():
            m.fit(ds, size_ratio=w.dim1, n_iter_max=1, n_iter_parafac=1, do_conv=False,
                  do_rwr=True, do_col=False, tol=0, run_init=False)
        if on_gpu:
            torch.cuda.synchronize()
        return m, time.perf_counter() - t0

    def init_state(w, ds):
        m, _ = one_fit(w, ds, None)
        return ([a.clone() for a in m.A_list], {k: v.clone() for k, v in m.B_dict.items()},
                {k: v.clone() for k, v in m.D_dict.items()}, m.meta_embedding.clone(),
                np.array(m.n_i).copy(), list(m.bin_cov_list), list(m.bad_bin_cov_list))

    w, ds = sample(n_cells)
    state = init_state(w, ds)
    times = []
    for i in range(warmup + steps):
        _, t = one_fit(w, ds, state)
        if i >= warmup:
            times.append(t)
    t_full = float(np.median(times))
    wh, dsh = sample(max(w.rank, n_cells // 2))
    st_h = init_state(wh, dsh)
    half = []
    for i in range(warmup + steps):
        _, t = one_fit(wh, dsh, st_h)
        if i >= warmup:
            half.append(t)
    t_half = float(np.median(half))
    per_cell = max((t_full - t_half) / (w.n_cells - wh.n_cells), 0.0)
    fixed = max(t_full - per_cell * w.n_cells, 0.0)
    fit_s = iters * (fixed + per_cell * w_full.n_cells)
    rate = w_full.n_cells / fit_s
    if on_gpu:
        return rate, t_full, {
            "kind": "reference", "device": torch.cuda.get_device_name(cpu), "extrapolated": True,
            "sample_cells": w.n_cells, "sample_iters": 1,
            "measured_s": [round(t, 3) for t in times], "half_sample_cells": wh.n_cells,
            "half_sample_s": round(t_half, 3), "fixed_s_per_iter": round(fixed, 4),
            "per_cell_s_per_iter": round(per_cell, 7), "stand_ins": notes,
            "sample": ("the reference's Fast_Higashi_core.fit with its torch path on this GPU, "
                       "one ALS iteration (with its RWR recomputations) per step on %d of %d "
                       "cells, from the reference's own init; one more at %d cells; extrapolated "
                       "to %d iterations x %d cells" % (w.n_cells, w_full.n_cells, wh.n_cells,
                                                         iters, w_full.n_cells))}
    desc = {"kind": "reference", "cores": threads, "extrapolated": True,
            "sample_cells": w.n_cells, "sample_iters": 1, "measured_s": [round(t, 3) for t in times],
            "half_sample_cells": wh.n_cells, "half_sample_s": round(t_half, 3),
            "fixed_s_per_iter": round(fixed, 4), "per_cell_s_per_iter": round(per_cell, 6),
            "rwr_epochs": sorted(set(int(v) for v in state[4])), "stand_ins": notes,
            "sample": ("the reference's Fast_Higashi_core.fit on the host CPU (%d threads), one "
                       "ALS iteration (with its RWR recomputations) per step on %d of %d cells, "
                       "from the reference's own init; one more at %d cells separates the "
                       "per-iteration cost that does not grow with cells; extrapolated to %d "
                       "iterations x %d cells" % (threads, w.n_cells, w_full.n_cells,
                                                 wh.n_cells, iters, w_full.n_cells))}
    return rate, t_full, desc


def fp64_check(w, coo, state, n_i, iters, dev, embeddings):
    """Both forms' final meta embedding against an FP64 fit of the same workload from the same
    initial state and RWR epochs (tests/fp64_reference.py: the reference's fit loop in torch
    float64 on this GPU, pinned to the numpy oracle by the CPU tests), after an orthogonal
    Procrustes rotation.  Untimed; runs after every timed region."""
    import torch
    from fh_gb300 import synth
    tests = os.path.join(ROOT, "tests")
    if tests not in sys.path:
        sys.path.insert(0, tests)
    import fp64_reference as F
    bsb = [synth.recommend_batches(w, nb, w.n_cells)[0] for nb in w.chrom_bins]
    datas = F.chrom_datas(coo, w.chrom_names, bsb, [w.n_cells] * len(bsb), w.band)
    A0 = [a.detach().cpu().numpy() for a in state[0]]
    B0 = {k: v.detach().cpu().numpy() for k, v in state[1].items()}
    D0 = {k: v.detach().cpu().numpy() for k, v in state[2].items()}
    E0 = state[3].detach().cpu().numpy()
    t0 = time.perf_counter()
    ref = F.FP64Fit(datas, w.rank, A0, B0, D0, E0, [int(v) for v in n_i], dev).fit(iters)
    E64 = ref.E.cpu().numpy()
    secs = time.perf_counter() - t0
    del ref
    torch.cuda.empty_cache()
    out = {"aligned_embedding_error_vs_fp64": {k: F.aligned_error(v.detach().cpu().numpy(), E64)
                                               for k, v in embeddings.items()},
           "target": 1e-3, "fp64_fit_seconds": round(secs, 1), "iterations": iters,
           "yardstick": "the reference's fit loop in torch float64 on this GPU, same initial "
                        "state and RWR epochs (tests/fp64_reference.py)"}
    out["meets_target"] = all(v <= 1e-3 for v in out["aligned_embedding_error_vs_fp64"].values())
    return out


def bench_config(w, rows, iters, ws):
    """The config object both arms print (the same workload, so the same dict)."""
    return {"workload": "%s: %d cells, %d bins, R=%d, band %d, %d ALS iterations" %
                        (w.name, w.n_cells, sum(w.chrom_bins), w.rank, w.band, iters),
            "l2": "inputs larger than L2 (X: %d cells x %d band rows, %.1f GB in fp32)" %
                  (w.n_cells, rows, w.n_cells * rows * 4 / 1e9),
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def band_rows(w):
    """Band rows (bin-batch rows x compact columns, summed) of a workload: the X row count."""
    from fh_gb300 import synth
    total = 0
    for nb in w.chrom_bins:
        bsb, _ = synth.recommend_batches(w, nb, w.n_cells)
        for r0 in range(0, nb, bsb):
            rows = min(bsb, nb - r0)
            lo, hi = max(0, r0 - w.band), min(nb, r0 + rows + w.band)
            total += rows * (hi - lo)
    return total


def reference_arm(args, rank, ws):
    if rank != 0:
        return
    from fh_gb300 import synth
    w = synth.workload(args.config)
    iters = args.iters or w.n_iter
    line = {"metric": METRIC, "impl": "reference"}
    try:
        v, t_step, desc = reference_fit_rate(args.config, args.sample_cells, iters, args.steps,
                                             args.warmup)
    except (ImportError, FileNotFoundError, OSError) as e:
        line["unavailable"] = "the reference could not be imported: %s" % e
        print(json.dumps(line), flush=True)
        return
    line.update({"value": v, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
                 "warmup": args.warmup, "ms_per_step": 1000.0 * t_step,
                 "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "dtype": "f32", "data": "synthetic (seeded generator, %s)" % args.config,
                 "config": bench_config(w, band_rows(w), iters, ws),
                 "cpu_baseline": dict(desc, value=v, unit="cells/s"),
                 "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0}})
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------
def _raw_cells_device(idx, val, n_cells, dev):
    """One chromosome's contacts as raw per-cell arrays on the device (cell-major, each cell's
    entries in (row, col) order; values expm1 of the packed ones, positive), built with torch
    outside every timed region."""
    import torch
    ii = torch.from_numpy(idx).to(dev)
    cell, perm = torch.sort(ii[2].long(), stable=True)
    row = ii[0][perm].contiguous()
    col = ii[1][perm].contiguous()
    v = torch.expm1(torch.from_numpy(val).to(dev)[perm]).contiguous()
    off = torch.zeros(n_cells + 1, dtype=torch.int64, device=dev)
    off[1:] = torch.cumsum(torch.bincount(cell, minlength=n_cells), 0)
    return row, col, v, off


def pack_measure(w, coo, dev, reps=3, sample_cells=300):
    """Input packing (fh_pack_chromosome, FastHigashi_Wrapper.py:221-366) of every chromosome
    of the workload from raw per-cell contacts resident in HBM, device-timed (median of reps
    per chromosome, summed); algorithmic traffic 28 B per contact (row, col, value read once;
    row, col, cell, value written once).  Beside it, the oracle's packing (NumPy, one host
    thread) of the first sample_cells cells of the first chromosome, scaled per contact."""
    import torch
    from fh_gb300 import _lib
    from oracle import fh_oracle as O
    P = _lib.ptr
    C = w.n_cells
    order = torch.arange(C, dtype=torch.int32, device=dev)
    total_ms, contacts = 0.0, 0
    for (idx, val, shape), nb in zip(coo, w.chrom_bins):
        row, col, v, off = _raw_cells_device(idx, val, C, dev)
        n = int(v.numel())
        out_idx = torch.empty((3, n), dtype=torch.int32, device=dev)
        out_val = torch.empty(n, dtype=torch.float32, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        ws_ = torch.empty(_lib.value("fh_pack_workspace", C, nb, 1, n), dtype=torch.uint8,
                          device=dev)
        a = (P(row), P(col), P(v), P(off), C, P(order), C, nb, 1, w.band, P(out_idx), P(out_val),
             n, P(counts), P(ws_), ws_.numel(), P(st), _lib.stream_ptr())
        _lib.call("fh_pack_chromosome", *a)
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.call("fh_pack_chromosome", *a)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        if int(st.item()) != 0 or int(counts[0].item()) != n:
            raise RuntimeError("packing check failed")
        total_ms += float(np.median(times))
        contacts += n
        del row, col, v, off, out_idx, out_val, ws_
    torch.cuda.empty_cache()
    hbm = peaks()[0]
    gbs = 28.0 * contacts / (total_ms / 1000.0) / 1e9
    # the oracle on a sample of the first chromosome's cells (host)
    idx, val, _ = coo[0]
    keep = idx[2] < sample_cells
    r, c, k, vv = idx[0][keep], idx[1][keep], idx[2][keep], np.expm1(val[keep])
    o = np.argsort(k, kind="stable")
    bounds = np.searchsorted(k[o], np.arange(sample_cells + 1))
    cells = [(r[o][bounds[i]:bounds[i + 1]], c[o][bounds[i]:bounds[i + 1]],
              vv[o][bounds[i]:bounds[i + 1]]) for i in range(sample_cells)]
    t0 = time.perf_counter()
    O.pack_chromosome(cells, w.chrom_bins[0], np.arange(sample_cells), w.band)
    cpu_s = time.perf_counter() - t0
    cpu_rate = int(keep.sum()) / cpu_s
    return {"what": "fh_pack_chromosome over all %d chromosomes, %d cells, raw contacts "
                    "resident in HBM (device time, median of %d per chromosome)"
                    % (len(coo), C, reps, ),
            "contacts": contacts, "ms": round(total_ms, 3),
            "contacts_per_s": contacts / (total_ms / 1000.0),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                         "frac": gbs / hbm, "work": "28 B per contact"},
            "cpu_baseline": {"kind": "port", "cores": 1, "contacts_per_s": cpu_rate,
                             "sample": "the oracle's pack_chromosome on the first %d cells of "
                                       "%s (%d contacts), one host thread"
                                       % (sample_cells, w.chrom_names[0], int(keep.sum())),
                             "extrapolated_s": contacts / cpu_rate}}


def postprocess_measure(w, E, D_list, dev, reps=3, sample_cells=1000):
    """fetch_cell_embedding + correct_batch_linear (FastHigashi_Wrapper.py:750-878) on the GPU
    for every cell (the embedding, the quantile transform, both truncated SVDs, the regression,
    the row normalisations), device-timed; the oracle (NumPy, fp64, exact SVDs) on a sample of
    cells beside it, scaled per cell."""
    import torch
    from fh_gb300.postprocess import (cell_embedding, quantile_transform_uniform,
                                      linear_residual, truncated_svd_in_span, l2_normalize)
    from oracle import fh_oracle as O
    C, R = E.shape
    rc = np.round(np.exp(np.random.default_rng(7).normal(11, 0.8, C)))

    def chain():
        Y = cell_embedding(E, D_list, dev)
        cov = quantile_transform_uniform(rc, 100, dev)
        emb, _ = truncated_svd_in_span(E, Y, R, dev)
        l2_normalize(emb, dev)
        res = linear_residual(cov.reshape(-1, 1), Y, False, dev)
        F = torch.cat([E, cov.reshape(-1, 1).float(),
                       torch.ones((C, 1), dtype=torch.float32, device=dev)], dim=1)
        red, _ = truncated_svd_in_span(F, res, R, dev)
        return l2_normalize(red, dev)

    chain()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        chain()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    Eh = E[:sample_cells].cpu().numpy()
    Dh = [d.cpu().numpy() for d in D_list]
    t0 = time.perf_counter()
    st = O.fetch_cell_embedding(Eh, Dh, rc[:sample_cells], R)
    cpu_s = time.perf_counter() - t0
    return {"what": "embedding, quantile transform, truncated SVD, coverage regression and its "
                    "truncated SVD, row normalisation, for %d cells x %d columns (device time, "
                    "median of %d)" % (C, st["embed_all"].shape[1], reps),
            "ms": round(ms, 3), "cells_per_s": C / (ms / 1000.0),
            "cpu_baseline": {"kind": "port", "cores": os.cpu_count(),
                             "cells_per_s": sample_cells / cpu_s,
                             "sample": "the oracle's fetch_cell_embedding (with its coverage "
                                       "regression) on %d cells, NumPy fp64" % sample_cells}}


def extras_arm(args, local):
    """The rows either side of the fit on their own: init_params (for E and D), then the input
    packing and post-processing measurements."""
    import torch
    from fh_gb300 import Fast_Higashi_core
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    w, coo, ds = make_workload(args.config, cells=args.cells)
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution], precision=args.precision).to(dev)
    m._sizes(ds, w.dim1, None)
    m.init_params(ds, False, True, False, seed=0)
    torch.cuda.synchronize()
    m.engine = None
    torch.cuda.empty_cache()
    line = {"workload": "%s: %d cells, %d bins, R=%d" % (w.name, w.n_cells, sum(w.chrom_bins),
                                                        w.rank),
            "input_packing": pack_measure(w, coo, dev),
            "post_processing": postprocess_measure(w, m.meta_embedding[:, :w.rank].contiguous(),
                                                   [m.D_dict[d.chrom] for d in ds], dev)}
    print(json.dumps(line), flush=True)


def budget_arm(args, rank, local, ws):
    """A workload whose X is larger than the HBM budget (c5: 50,000 cells at 500 kb, R = 128,
    band 40; X is 179 GB in two bf16 planes or in fp32): both forms run with hbm_budget, so
    X's last chromosomes stream through two staging slots from page-locked host memory and the
    contact segments are built one dataset at a time from the host COO (in page-locked
    memory), copied in chunks through the staging area.  A step is a whole fit: the contact
    build and walk (the COO crosses the host link inside the step)
    and the 30 ALS iterations (one CUDA graph, the window copies as memcpy nodes).  The COO is
    generated on the GPU (synth.generate_on_device) and kept in host memory, as a caller's
    input would be.  No end-to-end line beyond the step itself (its input already comes from
    host memory), no FP64 fit at this size (run --config c5 --cells 2000 for the precision
    report on the same shapes)."""
    import dataclasses
    import gc
    import torch
    from fh_gb300 import Fast_Higashi_core, _lib, synth
    from fh_gb300.engine import FitEngine
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    budget = int(args.hbm_budget_gb * 1e9)
    w = synth.workload(args.config)
    if args.cells:
        w = dataclasses.replace(w, n_cells=int(args.cells),
                                name="%s at %d cells" % (args.config, args.cells))
    iters = args.iters or w.n_iter
    C = w.n_cells
    t0 = time.time()
    coo, _ = synth.generate_on_device(w, seed=0, device=dev, pinned=True)
    gen_s = time.time() - t0
    ds = []
    for (idx, val, shape), cname, nb in zip(coo, w.chrom_names, w.chrom_bins):
        bsb, bsc = synth.recommend_batches(w, nb, w.n_cells)
        ds.append(Chrom_Dataset(Sparse(idx, val, shape, copy=False), bsb, bsc, compact=True,
                                flank=w.band, chrom=cname, resolution=w.resolution))
    nnz = int(sum(v.size for _, v, _ in coo))
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats(dev)
    torch.manual_seed(0)
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution], precision=args.precision,
                          hbm_budget=budget).to(dev)
    m._sizes(ds, w.dim1, None)
    t0 = time.time()
    m.init_params(ds, False, True, False, seed=0)
    torch.cuda.synchronize()
    init_s = time.time() - t0
    state = ([a.clone() for a in m.A_list], {k: v.clone() for k, v in m.B_dict.items()},
             {k: v.clone() for k, v in m.D_dict.items()}, m.meta_embedding.clone())
    n_i = np.asarray(m.n_i).copy()
    chrom2size = dict(m.chrom2size)

    def device_step(e, h, graph=True):
        e.run_rwr()
        e.set_state(*state)
        e.core_norm()
        e.run_iterations(iters, 1, h, graph=graph)

    def timed(e, h, warmup, steps, clocks):
        for _ in range(warmup):
            device_step(e, h)
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0, l0, c0 = _lib.launches, e.xs.link_bytes, e.store.link_bytes
        with Clocks(local) if clocks else _Null() as clk:
            torch.cuda.synchronize()
            s0.record()
            for _ in range(steps):
                device_step(e, h)
            s1.record()
            torch.cuda.synchronize()
        e.check_status("bench")
        return (s0.elapsed_time(s1) / steps, (_lib.launches - n0) // steps,
                ((e.xs.link_bytes - l0) / steps, (e.store.link_bytes - c0) / steps), clk)

    def plan_of(e):
        p = e.xs.plan
        return {"resident_gb": round(p.res_bytes / 1e9, 2),
                "streamed_gb": round(p.streamed_bytes / 1e9, 2),
                "windows": [{"chromosomes": [w.chrom_names[c] for c in win.chroms],
                             "gb": round(win.nbytes / 1e9, 2)} for win in p.windows],
                "staging_gb": round(p.staging_bytes / 1e9, 2)}

    eng = m.engine
    hist = eng.new_history(iters)
    ms, launches, (win_bytes, coo_bytes), clk = timed(eng, hist, args.warmup, args.steps, True)
    eng.timing = {}
    device_step(eng, hist, graph=False)
    torch.cuda.synchronize()
    summ = eng.timing_summary()
    kt = {k: round(v["mean_ms"], 3) for k, v in summ.items()}
    if "contacts" in summ:            # per dataset; the step's total beside it
        kt["contacts_per_step"] = round(summ["contacts"]["total_ms"], 3)
    eng.timing = None
    E_main = eng.E[:, :w.rank].clone()
    loss = float(eng.losses(hist[-1], eng.tensor_norms())[0])
    peak = torch.cuda.max_memory_reserved(dev)
    free, total = torch.cuda.mem_get_info(dev)
    mem = {"budget_gb": budget / 1e9, "peak_reserved_gb": round(peak / 1e9, 2),
           "device_used_gb_after": round((total - free) / 1e9, 2)}
    main_plan = plan_of(eng)
    link = {"coo_copied_gb": round(coo_bytes / 1e9, 2),
            "window_copies_gb": round(win_bytes / 1e9, 2)}
    del m, eng, hist
    gc.collect()
    torch.cuda.empty_cache()
    plain = None
    if args.precision != "fp32" and not args.no_plain:
        torch.cuda.reset_peak_memory_stats(dev)
        peng = FitEngine(ds, w.rank, chrom2size, n_i, dev, precision="fp32", hbm_budget=budget)
        phist = peng.new_history(iters)
        pms, plaunch, (pwin, _), _ = timed(peng, phist, args.warmup, args.steps, False)
        plain = {"value": C / (pms / 1000.0), "unit": "cells/s", "ms_per_step": pms,
                 "gpu_launches": int(plaunch), "speedup_of_headline": pms / ms,
                 "embedding_aligned_rel_diff": aligned_diff(E_main, peng.E[:, :w.rank]),
                 "peak_reserved_gb": round(torch.cuda.max_memory_reserved(dev) / 1e9, 2),
                 "x_plan": plan_of(peng), "window_copies_gb": round(pwin / 1e9, 2)}
        del peng, phist
        gc.collect()
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": C / (ms / 1000.0), "unit": "cells/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16" if args.precision != "fp32" else "fp32",
            "data": "synthetic (seeded generator on the GPU, %s)" % args.config,
            "config": {"workload": "%s: %d cells, %d bins, R=%d, band %d, %d ALS iterations" %
                                   (w.name, C, sum(w.chrom_bins), w.rank, w.band, iters),
                       "contacts": nnz, "hbm_budget_gb": budget / 1e9,
                       "l2": "inputs larger than L2 (X %.0f GB)" % (C * band_rows(w) * 4 / 1e9),
                       "parallelism": "single GPU"},
            "precision": args.precision, "rwr_epochs": [int(v) for v in n_i],
            "memory": mem, "x_plan": main_plan, "host_link_per_step": link,
            "kernel_ms": kt, "gpu_launches": int(launches), "clocks": clk.summary(),
            "plain_fp32": plain, "loss_final": loss,
            "setup_s": {"generate": round(gen_s, 1), "init_params": round(init_s, 1)}}))
        sys.stdout.flush()


def gb300_arm(args, rank, local, ws):
    import torch
    from fh_gb300 import Fast_Higashi_core, _lib
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    w, coo, ds = make_workload(args.config, cells=args.cells)
    iters = args.iters or w.n_iter
    C = w.n_cells
    # ---- init (untimed): the GPU init_params, then the state every step starts from
    torch.manual_seed(0)
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution], precision=args.precision).to(dev)
    m._sizes(ds, w.dim1, None)
    m.init_params(ds, False, True, False, seed=0)
    torch.cuda.synchronize()
    state = ([a.clone() for a in m.A_list], {k: v.clone() for k, v in m.B_dict.items()},
             {k: v.clone() for k, v in m.D_dict.items()}, m.meta_embedding.clone())
    eng = m.engine
    hist = eng.new_history(iters)

    def device_step(e, h, graph=True):
        e.store.rebuild()
        e.run_rwr()
        e.set_state(*state)
        e.core_norm()
        e.run_iterations(iters, 1, h, graph=graph)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    def timed(e, h, clocks):
        """W warm-up fits, then K fits bracketed by a barrier and synchronizes; max over ranks."""
        for _ in range(args.warmup):
            device_step(e, h)
        torch.cuda.synchronize()
        barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = _lib.launches
        with Clocks(local) if clocks else _Null() as clk:
            torch.cuda.synchronize()
            s0.record()
            for _ in range(args.steps):
                device_step(e, h)
            s1.record()
            torch.cuda.synchronize()
        n_launch = (_lib.launches - n0) // args.steps
        t = max_over_ranks(torch.tensor([s0.elapsed_time(s1) / args.steps], device=dev), ws)
        e.check_status("bench")
        return float(t.item()), n_launch, clk

    ms, launches, clk = timed(eng, hist, True)
    value = ws * C / (ms / 1000.0)
    # ---- end to end through the public API, host data in and out (before the plain form, so
    # that each measurement starts from the same device state: this engine and nothing else)
    A0, B0, D0, E0 = [x.cpu() for x in state[0]], {k: v.cpu() for k, v in state[1].items()}, \
        {k: v.cpu() for k, v in state[2].items()}, state[3].cpu()
    n_i = m.n_i.copy()

    store_h2d = [0]

    def e2e_step():
        mm = Fast_Higashi_core(w.rank, w.band, [w.resolution], precision=args.precision).to(dev)
        mm._sizes(ds, w.dim1, None)
        mm.A_list, mm.B_dict, mm.D_dict, mm.meta_embedding = A0, B0, D0, E0
        mm.n_i, mm.bin_cov_list = n_i, [None] * len(ds)
        mm.fit(ds, size_ratio=w.dim1, n_iter_max=iters, n_iter_parafac=1, do_conv=False,
               do_rwr=True, do_col=False, tol=0, run_init=False, verbose=False)
        emb = mm.meta_embedding.cpu()
        store_h2d[0] = mm.engine.store.h2d_bytes
        del mm                       # the next step's engine reuses the freed device memory
        return emb

    e2e_step()
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(max(2, args.steps)):
        barrier()
        t0 = time.perf_counter()
        emb = e2e_step()
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = float(np.median(e2e_times))     # each step is a whole fit through the public API
    e2e_s = float(max_over_ranks(torch.tensor([e2e_s], device=dev), ws).item())
    h2d = store_h2d[0] + sum(a.numel() * 4 for a in A0) + E0.numel() * 4 + \
        sum(v.numel() * 4 for v in B0.values()) + sum(v.numel() * 4 for v in D0.values())
    d2h = emb.numel() * 4 + iters * (eng.nb + 1 + len(eng.names)) * 8
    e2e = {"value": ws * C / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1000.0,
           "ms_steps": [round(t * 1000.0, 1) for t in e2e_times], "statistic": "median"}
    # ---- the plain fp32 form on the same state, for the BF16-batched vs plain FP32 ratio
    plain = None
    if args.precision != "fp32" and not args.no_plain:
        from fh_gb300.engine import FitEngine
        peng = FitEngine(ds, w.rank, m.chrom2size, m.n_i, dev, precision="fp32")
        phist = peng.new_history(iters)
        pms, plaunch, _ = timed(peng, phist, False)
        peng.timing = {}
        device_step(peng, phist, graph=False)
        torch.cuda.synchronize()
        pkt = peng.timing_summary()
        E_plain = peng.E[:, :w.rank].clone()
        plain = {"value": ws * C / (pms / 1000.0), "unit": "cells/s", "ms_per_step": pms,
                 "gpu_launches": int(plaunch),
                 "kernel_ms": {k: round(v["mean_ms"], 4) for k, v in pkt.items()},
                 "speedup_of_headline": (ws * C / (ms / 1000.0)) / (ws * C / (pms / 1000.0)),
                 "embedding_aligned_rel_diff": aligned_diff(eng.E[:, :w.rank], peng.E[:, :w.rank]),
                 "loss_final": float(peng.losses(phist[-1], peng.tensor_norms())[0])}
        del peng
        torch.cuda.empty_cache()
    # ---- per-kernel times (one instrumented step) for the roofline
    eng.timing = {}
    device_step(eng, hist, graph=False)
    torch.cuda.synchronize()
    kt = eng.timing_summary()
    eng.timing = None
    xel = 2 * eng.planes if eng.bf16 else 4
    from fh_gb300.engine import FitEngine
    fams = family_rooflines(eng, kt, clk.summary().get("sm_max_mhz"),
                            FitEngine.parafac_schedule(iters, 1))
    share = {k: round(v["total_ms"] / ms, 3) for k, v in kt.items()}
    dom = max(fams, key=lambda f: kt[f["kernel"]]["total_ms"])
    roof = dict(dom)
    if dom["kernel"] in ("xe", "xg") and eng.precision == "bf16x2":
        roof["traffic"] = XPASS_TRAFFIC_RATIO[dom["kernel"]] * dom["work_per_launch"] / 1e9
        roof["traffic_unit"] = "GB per launch (ncu at 2,000 cells, scaled by cells x band rows)"
    elif dom["kernel"] == "procrustes":
        roof["traffic"] = PROCRUSTES_TRAFFIC_PER_ROW * eng.nb / 1e9
        roof["traffic_unit"] = "GB per launch (ncu at 2,000 cells, scaled by bin rows)"
    else:
        roof["traffic"] = None
    roof["note"] = ("the family with the largest share of the step; every family in families, "
                    "shares of the step: %s" % share)
    roof["families"] = fams
    # ---- the rows either side of the fit: input packing and post-processing (untimed by the
    # headline; each device-timed on its own)
    packing = post = None
    if not args.no_extras and rank == 0:
        packing = pack_measure(w, coo, dev)
        post = postprocess_measure(w, m.meta_embedding[:, :w.rank].contiguous(),
                                   [m.D_dict[d.chrom] for d in ds], dev)
    # ---- both forms' error against an FP64 fit from the same state (untimed)
    precision = None
    if not args.no_fp64:
        embs = {eng.precision: eng.E[:, :w.rank].clone()}
        if plain is not None:
            embs["fp32"] = E_plain
        precision = fp64_check(w, coo, state, n_i, iters, dev, embs)
    if rank != 0:
        return
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        try:
            r, _, desc = reference_fit_rate(args.config, args.sample_cells, iters, 2, 1)
            cpu = dict(desc, value=r, unit="cells/s")
        except (ImportError, FileNotFoundError, OSError) as e:
            cpu = {"unavailable": "the reference could not be imported: %s" % e}
    # context, not a baseline: the reference's own torch path on this GPU (what a current user
    # of the reference sees), on a larger cell sample
    ref_gpu = None
    if ws == 1 and not args.no_cpu_baseline and not args.no_reference_gpu:
        try:
            r, _, desc = reference_fit_rate(args.config, args.gpu_sample_cells, iters, 2, 1,
                                            device="cuda")
            ref_gpu = dict(desc, value=r, unit="cells/s")
        except Exception as e:          # reported, never fatal to the line
            ref_gpu = {"unavailable": "%s: %s" % (type(e).__name__, str(e)[:200])}
        torch.cuda.empty_cache()
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16" if eng.bf16 else "f32",
            "data": "synthetic (seeded generator, %s)" % args.config,
            "config": bench_config(w, eng.rows, iters, ws),
            "precision": ({"bf16": "X in one bf16 plane, tensor-core X passes",
                           "bf16x2": "X in two bf16 planes (hi+lo), tensor-core X passes"}
                          .get(eng.precision, "fp32 (plain)")),
            "rwr_epochs": sorted(set(int(v) for v in n_i)), "bin_batches": eng.n_tiles,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "reference_gpu": ref_gpu, "plain_fp32": plain,
            "clocks": clk.summary(), "kernel_ms": {k: round(v["mean_ms"], 4) for k, v in kt.items()},
            "autotune": autotune_summary(), "precision_check": precision,
            "input_packing": packing, "post_processing": post,
            "loss_final": float(m.engine.losses(hist[-1], eng.tensor_norms())[0])}
    print(json.dumps(line), flush=True)


def grad_arm(args, rank, local, ws):
    """Forward + backward of the per-cell reconstruction loss (fh_gb300.differentiable) on a
    fitted state: the RWR at rp, the Gt rows and the fused loss; then the recomputed RWR with
    its rp-derivative, the fused residual backward, U^T dGt and the factor gradients."""
    import torch
    from fh_gb300 import Fast_Higashi_core, _lib
    from fh_gb300.differentiable import ReconstructionLoss
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    w, coo, ds = make_workload(args.config, cells=args.cells)
    torch.manual_seed(0)
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution]).to(dev)
    m.fit(ds, size_ratio=w.dim1, n_iter_max=args.iters or 3, n_iter_parafac=1, do_conv=False,
          do_rwr=True, do_col=False, tol=0, verbose=False)
    eng = m.engine
    layer = ReconstructionLoss(m)
    leaves = [m.meta_embedding.detach().clone()] + [a.detach().clone() for a in m.A_list] + \
        [m.B_dict[d.chrom].detach().clone() for d in ds] + [m.D_dict[d.chrom].detach().clone() for d in ds]
    for t in leaves:
        t.requires_grad_()
    n = len(ds)
    rp = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)

    def step():
        loss = layer(rp, leaves[0], leaves[1:1 + n], leaves[1 + n:1 + 2 * n], leaves[1 + 2 * n:])
        loss.sum().backward()
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = _lib.launches
    with Clocks(local) as clk:
        s0.record()
        for _ in range(args.steps):
            step()
        s1.record()
        torch.cuda.synchronize()
    ms = s0.elapsed_time(s1) / args.steps
    launches = (_lib.launches - n0) // args.steps
    layer.timing = {}
    step()
    torch.cuda.synchronize()
    kt = layer.timing_summary()
    layer.timing = None
    # algorithmic flops (fp32 FMA work) per kernel family
    t = eng.tiles
    b, nw, ep = t["rows"].astype(float), t["width"].astype(float), t["n_rwr"].astype(float)
    C, Ct, R = eng.C, eng.Ct, w.rank
    fl = {"rwr_rp": Ct * float((2 * b * b * nw * (1 + ep)).sum()),
          "rwr_grad": Ct * float((2 * b * b * nw * (1 + 2 * ep)).sum()),
          "recon_loss": 2.0 * eng.rows * C * R,
          "recon_bwd": 8.0 * eng.rows * C * R}
    clock = clk.summary()
    mhz = clock.get("sm_max_mhz") or 2070.0
    fp32_peak = 2 * 128 * 152 * mhz * 1e6 / 1e12    # nominal fp32 CUDA-core TFLOP/s
    fam = max(fl, key=lambda k: kt.get(k, {}).get("total_ms", 0))
    ach = fl[fam] / (kt[fam]["mean_ms"] / 1000.0) / 1e12
    kernels = {k: {"ms": round(v["mean_ms"], 3),
                   "tflops": round(fl[k] / (v["mean_ms"] / 1000.0) / 1e12, 2) if k in fl else None}
               for k, v in kt.items()}
    if rank != 0:
        return
    line = {"metric": "differentiable reconstruction loss, forward + backward (rp, E, A, B, D)",
            "value": ms, "unit": "ms per forward+backward", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, %s)" % args.config,
            "config": {"workload": "%s: %d cells, %d bins (%d bin batches), R=%d, band %d, fitted "
                                   "state after %d ALS iterations" %
                                   (w.name, C, sum(w.chrom_bins), eng.n_tiles, R, w.band,
                                    args.iters or 3),
                       "l2": "inputs larger than L2 (X %.2f GB fp32)" % (Ct * eng.ldx * 4 / 1e9)},
            "roofline": {"kernel": fam, "bound": "fp32", "achieved": ach, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": ach / fp32_peak,
                         "peak_kind": "nominal fp32 CUDA-core rate at the sampled maximum clock",
                         "traffic": None},
            "kernels": kernels, "gpu_launches": int(launches), "clocks": clock}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, local, ws = dist_setup()
    if args.grad:
        from fh_gb300 import build as _b
        _b.build()
        grad_arm(args, rank, local, ws)
    elif args.impl == "reference":
        reference_arm(args, rank, ws)
    elif args.extras_only:
        from fh_gb300 import build as _b
        _b.build()
        if rank == 0:
            extras_arm(args, local)
    elif args.hbm_budget_gb is not None:
        from fh_gb300 import build as _b
        _b.build()
        budget_arm(args, rank, local, ws)
    else:
        from fh_gb300 import build as _b
        _b.build()
        gb300_arm(args, rank, local, ws)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
