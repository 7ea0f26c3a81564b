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
  --impl reference   the CPU restatement of the reference (the oracle, fp32, all host threads)
                     on a bounded cell sample, extrapolated to cells/s

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
    ap.add_argument("--sample-cells", type=int, default=96,
                    help="cells of the CPU-baseline sample (at least the rank R)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="bf16x2", choices=["fp32", "bf16x2", "bf16"],
                    help="form timed for the headline: bf16x2 (default) the tensor-core form, X "
                         "as two bf16 planes; bf16 one plane; fp32 the plain drop-in")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip timing the plain fp32 form beside the headline form")
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
    # The generator fills each chromosome's arrays in its own worker thread; copy them once in
    # this thread, as arrays read from a file by the caller would be allocated.  Untimed.
    coo = [(np.array(idx, copy=True), np.array(val, copy=True), shape) for idx, val, shape in coo]
    ds = []
    for (idx, val, shape), cname, nb in zip(coo, w.chrom_names, w.chrom_bins):
        bsb, bsc = synth.recommend_batches(w, nb, w.n_cells)
        ds.append(Chrom_Dataset(Sparse(idx, val, shape, copy=False), bsb, bsc, compact=True,
                                flank=w.band, chrom=cname, resolution=w.resolution))
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


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback"


# --------------------------------------------------------------------------------------
def cpu_sample_rate(coo, w, n_cells, iters, threads=None):
    """Cells/s of the CPU restatement (fp32, the reference's loop structure with its RWR
    recomputation) on the first n_cells cells: RWR + one warm ALS iteration, extrapolated
    to RWR + iters iterations.  Returns (cells/s, sample description, seconds spent)."""
    from oracle import fh_oracle as O
    from fh_gb300 import synth
    n_cells = max(n_cells, w.rank)
    t0 = time.perf_counter()
    datas = []
    for k, ((idx, val, shape), nb) in enumerate(zip(coo, w.chrom_bins)):
        m = idx[2] < n_cells
        bsb, _ = synth.recommend_batches(w, nb, w.n_cells)
        datas.append(O.ChromData("chr%d" % (k + 1), idx[:, m], val[m], nb, n_cells, bsb, n_cells, w.band))
    sizes = O.chrom2size(datas, w.rank, w.dim1, w.resolution)
    rng = np.random.default_rng(0)
    A = [1 + 0.01 * rng.standard_normal((d.num_bin, sizes[d.name])) for d in datas]
    B = {d.name: np.eye(sizes[d.name]) + 0.01 * rng.standard_normal(sizes[d.name]) for d in datas}
    D = {d.name: rng.standard_normal((w.rank, sizes[d.name])) for d in datas}
    E, _ = np.linalg.qr(rng.standard_normal((n_cells, w.rank)))
    orc = O.ALSOracle(datas, w.rank, A, B, D, E, [6] * len(datas), dtype=np.float32, cache_rwr=False)
    t = time.perf_counter()
    for ci, d in enumerate(datas):                       # the RWR pass of init / the first fetch
        for bi in range(len(d.layout())):
            orc.rwr_tile(ci, bi, 0)
    t_rwr = time.perf_counter() - t
    orc.iterate(0, 1)
    t = time.perf_counter()
    orc.iterate(1, 1)
    t_iter = time.perf_counter() - t
    rate = n_cells / (t_rwr + iters * t_iter)
    desc = ("%d of %d cells, RWR pass %.2fs + 1 timed ALS iteration %.2fs (3 RWR recomputations "
            "per bin batch, as the reference), extrapolated to %d iterations" %
            (n_cells, w.n_cells, t_rwr, t_iter, iters))
    return rate, desc, time.perf_counter() - t0


def reference_arm(args, rank, ws):
    if rank != 0:
        return
    w, coo, _ = make_workload(args.config, cells=args.cells)
    iters = args.iters or w.n_iter
    threads = os.cpu_count()
    rates, desc = [], ""
    for i in range(args.warmup + args.steps):
        r, desc, _ = cpu_sample_rate(coo, w, args.sample_cells, iters)
        if i >= args.warmup:
            rates.append(r)
    v = float(np.mean(rates))
    line = {"metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * w.n_cells / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, %s)" % args.config, "impl": "reference",
            "config": {"workload": "%s: %d cells, %d bins, R=%d, band %d, %d ALS iterations" %
                       (w.name, w.n_cells, sum(w.chrom_bins), w.rank, w.band, iters),
                       "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": "cells/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------
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
    hbm, bf16, peak_kind = peaks()
    xel = 2 * eng.planes if eng.bf16 else 4
    xbytes = C * eng.rows * xel
    fam = max(("xe", "xg"), key=lambda k: kt.get(k, {}).get("total_ms", 0))
    dom = max(kt, key=lambda k: kt[k]["total_ms"])
    ach = xbytes / (kt[fam]["mean_ms"] / 1000.0) / 1e9
    traffic = (XPASS_TRAFFIC_RATIO[fam] * xbytes / 1e9) if eng.precision == "bf16x2" else None
    roof = {"kernel": fam, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
            "frac": ach / hbm, "peak_kind": peak_kind, "traffic": traffic,
            "traffic_unit": "GB per launch (ncu at 2,000 cells, scaled by cells x band rows)",
            "algorithmic_bytes_per_launch": xbytes,
            "note": ("X pass (%d cells x %d band rows %s); kernel share of the step: %s; "
                     "largest family: %s" % (C, eng.rows, eng.precision,
                                             {k: round(v["total_ms"] / ms, 3) for k, v in kt.items()},
                                             dom))}
    # ---- end to end through the public API, host data in and out
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
    if rank != 0:
        return
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        r, desc, _ = cpu_sample_rate(coo, w, args.sample_cells, iters)
        cpu = {"value": r, "unit": "cells/s", "cores": os.cpu_count(), "kind": "port", "sample": desc}
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16" if eng.bf16 else "f32", "data": "synthetic (seeded generator, %s)" % args.config,
            "config": {"workload": "%s: %d cells, %d bins (%d bin batches), R=%d, band %d, %d ALS "
                                   "iterations, RWR epochs %s" %
                                   (w.name, C, sum(w.chrom_bins), eng.n_tiles, w.rank, w.band,
                                    iters, sorted(set(int(v) for v in n_i))),
                       "precision": ({"bf16": "X in one bf16 plane, tensor-core X passes",
                                      "bf16x2": "X in two bf16 planes (hi+lo), tensor-core X passes"}
                                     .get(eng.precision, "fp32 (plain)")),
                       "l2": "inputs larger than L2 (X %.2f GB)" % (eng.Ct * eng.ldx * xel / 1e9), "parallelism": "replicas" if ws > 1 else "single GPU"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "plain_fp32": plain,
            "clocks": clk.summary(), "kernel_ms": {k: round(v["mean_ms"], 4) for k, v in kt.items()},
            "autotune": autotune_summary(),
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
    else:
        from fh_gb300 import build as _b
        _b.build()
        gb300_arm(args, rank, local, ws)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
