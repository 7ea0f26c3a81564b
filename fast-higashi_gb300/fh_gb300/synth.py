"""Seeded synthetic single-cell Hi-C generator for the fit hot path.

There is no public dataset in reach, so the workloads are generated: per cell
and per chromosome, contact counts are Poisson draws with expectation

    lambda_ij  ~  (|i - j| + 1) ** (-alpha_c)  *  exp(gamma * s_{t,i} * s_{t,j})

on the band |i - j| <= band, where alpha_c is the cell's distance-decay
exponent and s_t a +-1 compartment labelling of cell type t (blocks of 5-20
bins, drawn independently per type).  Per-cell totals are log-normal and are
split across chromosomes by length.  The matrix is stored symmetric (both
triangles), as the reference's per-cell scipy matrices are.

The reference's per-chromosome packing is then restated
(``fasthigashi/FastHigashi_Wrapper.py:265-269`` off-diagonal filter,
``fasthigashi/preprocessing.py:137-142`` coverage normalisation with
scale = #bins / total, ``FastHigashi_Wrapper.py:358-364`` log1p and clip at
mean + 15 std).  Bin filtering (``preprocessing.py:474``) keeps every bin with
non-zero bulk coverage; every synthetic bin has coverage, so the mapping is the
identity and is not applied.

The output per chromosome is the reference's ``Sparse`` COO layout: indices
int32[3, nnz] = (row bin, column bin, cell), values float32[nnz], sorted by
(row, column, cell) so that ``Sparse.sort_indices`` takes its fast path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Human autosome lengths in Mb (chr1..chr22), as used for the genome-scale workloads.
HUMAN_AUTOSOMES_MB = [249, 243, 199, 191, 182, 171, 160, 146, 139, 134, 136,
                      134, 115, 108, 102, 91, 84, 81, 59, 65, 47, 51]


@dataclass
class Workload:
    name: str
    n_cells: int
    chrom_bins: list
    resolution: int
    band: int
    alpha: object            # float or (lo, hi) for a per-cell uniform draw
    median_total: float
    sigma: float
    n_types: int
    rank: int
    n_iter: int
    gamma: float = 0.35
    ultra_sparse_frac: float = 0.0
    ultra_sparse_max: int = 5000
    dim1: float = 0.6
    chrom_names: list = field(default_factory=list)

    def __post_init__(self):
        if not self.chrom_names:
            self.chrom_names = ["chr%d" % (i + 1) for i in range(len(self.chrom_bins))]


def genome_bins(resolution: int, lengths_mb=HUMAN_AUTOSOMES_MB):
    return [int(math.ceil(l * 1_000_000 / resolution)) for l in lengths_mb]


def workload(name: str) -> Workload:
    """The named workloads.

    ``c1``  200 cells, 3 chromosomes of 100/80/60 bins at 1 Mb, band 10, R=16, 10 iterations.
    ``c2``  2,000 cells, 22 autosomes at 1 Mb (2,887 bins), band 20, R=64, 30 iterations.
    ``c3``  10,000 cells, 22 autosomes at 500 kb (5,774 bins), band 30, R=64, 30 iterations.
    ``c4``  2,000 cells at 500 kb, band 20, R=32 (differentiation workload).
    ``c5``  50,000 cells at 500 kb, band 40, R=128, 5 % ultra-sparse cells.
    ``r128``  240 cells, 2 chromosomes of 440/300 bins at 500 kb, band 20, R=128 (ranks 128
              and 90: the rank-128 kernels at test size).
    ``tiny`` / ``small``  reduced cases for tests.
    """
    if name == "c1":
        return Workload("c1", 200, [100, 80, 60], 1_000_000, 10, 1.1, 20_000, 0.5, 0, 16, 10)
    if name == "c2":
        return Workload("c2", 2000, genome_bins(1_000_000), 1_000_000, 20, (0.9, 1.3),
                        100_000, 0.8, 8, 64, 30)
    if name == "c3":
        return Workload("c3", 10_000, genome_bins(500_000), 500_000, 30, (0.9, 1.3),
                        100_000, 0.8, 12, 64, 30)
    if name == "c4":
        return Workload("c4", 2000, genome_bins(500_000), 500_000, 20, (0.9, 1.3),
                        100_000, 0.8, 8, 32, 30)
    if name == "c5":
        return Workload("c5", 50_000, genome_bins(500_000), 500_000, 40, (0.9, 1.3),
                        150_000, 1.0, 12, 128, 30, ultra_sparse_frac=0.05)
    if name == "r128":
        return Workload("r128", 240, [440, 300], 500_000, 20, (0.9, 1.3), 30_000, 0.6, 4, 128, 3)
    if name == "small":
        return Workload("small", 96, [70, 45, 33], 1_000_000, 6, (0.9, 1.3), 6_000, 0.6, 3, 8, 4)
    if name == "tiny":
        return Workload("tiny", 24, [37, 20], 1_000_000, 4, 1.1, 1_500, 0.5, 2, 6, 3)
    raise KeyError(name)


def _compartments(rng, n_types, nbin):
    s = np.ones((max(n_types, 1), nbin))
    for t in range(n_types):
        pos, sign = 0, (1.0 if rng.random() < 0.5 else -1.0)
        while pos < nbin:
            L = int(rng.integers(5, 21))
            s[t, pos:pos + L] = sign
            sign = -sign
            pos += L
    return s


def _upper_band(nbin, band):
    """Upper-band positions (i, i+d), d = 0..band, enumerated d-major."""
    ii, dd = [], []
    for d in range(min(band, nbin - 1) + 1):
        ii.append(np.arange(nbin - d))
        dd.append(np.full(nbin - d, d))
    return np.concatenate(ii), np.concatenate(dd)


def _band_rowmajor(nbin, band):
    """Both-triangle band positions sorted by (row, col)."""
    rows = np.repeat(np.arange(nbin), 2 * band + 1)
    cols = rows + np.tile(np.arange(-band, band + 1), nbin)
    ok = (cols >= 0) & (cols < nbin)
    return rows[ok], cols[ok]


def _chromosome(w, nbin, rng, totals, alpha, types, genome, cell_chunk):
    """COO (indices, values, shape) of one chromosome for every cell."""
    C = w.n_cells
    s = _compartments(rng, w.n_types, nbin)
    ui, ud = _upper_band(nbin, w.band)
    P_up = len(ui)
    w_sym = np.where(ud > 0, 2.0, 1.0)
    rows, cols = _band_rowmajor(nbin, w.band)
    # index of each both-triangle band position in the upper-band enumeration
    doff = np.concatenate([[0], np.cumsum([nbin - d for d in range(min(w.band, nbin - 1) + 1)])])
    up_idx = doff[np.abs(cols - rows)] + np.minimum(rows, cols)
    counts = np.empty((C, P_up), dtype=np.uint16)
    logd = np.log(ud + 1.0)
    for c0 in range(0, C, cell_chunk):
        c1 = min(C, c0 + cell_chunk)
        lam = np.exp(-alpha[c0:c1, None] * logd[None, :])
        if w.n_types > 0:
            st = s[types[c0:c1]]                      # (chunk, nbin)
            lam *= np.exp(w.gamma * st[:, ui] * st[:, ui + ud])
        lam *= (totals[c0:c1, None] * nbin / genome) / lam.sum(1, keepdims=True)
        counts[c0:c1] = np.minimum(rng.poisson(lam), 65535).astype(np.uint16)
    cell_sum = counts.astype(np.float64) @ w_sym                 # both triangles
    scale = nbin / (cell_sum + 1e-15)
    band_counts = counts[:, up_idx].T                            # (P_band, C), rows sorted
    del counts
    p, cell = np.nonzero(band_counts)
    cnt = band_counts[p, cell].astype(np.float32)
    del band_counts
    vals = np.log1p(cnt * scale[cell].astype(np.float32)).astype(np.float32)
    if vals.size:
        m, sd = np.mean(vals), np.std(vals)
        vals = np.clip(vals, None, m + 15 * sd).astype(np.float32)
    idx = np.empty((3, p.size), dtype=np.int32)
    idx[0] = rows[p]
    idx[1] = cols[p]
    idx[2] = cell
    return idx, vals, (nbin, nbin, C)


def generate(w: Workload, seed: int = 0, cell_chunk: int = 2048, threads: int = 0):
    """Returns (list of (indices int32[3,nnz], values float32[nnz], shape), meta dict).

    The per-cell quantities come from one generator, each chromosome from its own child of
    the seed, so chromosomes are generated in parallel threads (NumPy's samplers release the
    GIL) with a result that does not depend on the thread count."""
    import concurrent.futures as cf
    import os
    ss = np.random.SeedSequence(seed)
    cell_ss, *chrom_ss = ss.spawn(1 + len(w.chrom_bins))
    rng = np.random.default_rng(cell_ss)
    C = w.n_cells
    totals = np.exp(rng.normal(math.log(w.median_total), w.sigma, C))
    if w.ultra_sparse_frac > 0:
        k = int(round(w.ultra_sparse_frac * C))
        idx = rng.choice(C, size=k, replace=False)
        totals[idx] = rng.uniform(0.2, 1.0, size=k) * w.ultra_sparse_max
    if isinstance(w.alpha, tuple):
        alpha = rng.uniform(w.alpha[0], w.alpha[1], C)
    else:
        alpha = np.full(C, float(w.alpha))
    types = rng.integers(0, max(w.n_types, 1), C)
    genome = float(sum(w.chrom_bins))
    n_thr = threads or min(len(w.chrom_bins), os.cpu_count() or 1)
    jobs = [(nbin, np.random.default_rng(cs)) for nbin, cs in zip(w.chrom_bins, chrom_ss)]
    with cf.ThreadPoolExecutor(max_workers=n_thr) as ex:
        out = list(ex.map(lambda j: _chromosome(w, j[0], j[1], totals, alpha, types, genome,
                                                cell_chunk), jobs))
    meta = dict(totals=totals, alpha=alpha, types=types)
    return out, meta


def recommend_batches(w: Workload, nbin: int, n_cells: int, avail_bytes: float = 280e9):
    """Bin-batch and cell-batch sizes by the reference's GPU rule
    (``FastHigashi_Wrapper.py:497-517``): bs_bin = ceil(n / ceil(n / rec)) with
    rec = min(max(int(15e6 / res), 128), 256); bs_cell from free memory / 48."""
    rec = min(max(int(15_000_000 / w.resolution), 128), 256)
    n_batch = max(math.ceil(nbin / rec), 1)
    bs_bin = math.ceil(nbin / n_batch)
    max_tensor = avail_bytes / (4 * 12)
    bs_cell = int(max_tensor / (bs_bin * (bs_bin + 2 * w.band)))
    nb = int(math.ceil(n_cells / bs_cell))
    bs_cell = int(math.ceil(n_cells / nb))
    return bs_bin, min(bs_cell, n_cells)


def generate_on_device(w: Workload, seed: int = 0, device="cuda", cell_chunk: int = 8192,
                       band_chunk: int = 2048, pinned: bool = False):
    """The same model as generate(), with the Poisson draws and the packing on the GPU.

    For the largest workload (50,000 cells at 500 kb, about 7e9 contacts, 112 GB of COO) the
    host generator's intermediates would not fit the host's memory next to its output and
    would take minutes; here each chromosome's counts, band layout and nonzeros are formed on
    the device (in chunks of cells and of band positions), and only the finished COO (int32
    indices, float32 values, sorted by row, column and cell) is copied into host arrays.  The
    per-cell quantities (totals, decay exponents, types) and each chromosome's compartments
    come from the same seeded NumPy generators as generate(); the draws come from torch's
    seeded CUDA generator, so the contacts are reproducible but differ from generate()'s.
    With pinned, the COO lands in page-locked host buffers (exact size), ready for copies."""
    import torch
    dev = torch.device(device)
    ss = np.random.SeedSequence(seed)
    cell_ss, *chrom_ss = ss.spawn(1 + len(w.chrom_bins))
    rng = np.random.default_rng(cell_ss)
    C = w.n_cells
    totals = np.exp(rng.normal(math.log(w.median_total), w.sigma, C))
    if w.ultra_sparse_frac > 0:
        k = int(round(w.ultra_sparse_frac * C))
        idx = rng.choice(C, size=k, replace=False)
        totals[idx] = rng.uniform(0.2, 1.0, size=k) * w.ultra_sparse_max
    if isinstance(w.alpha, tuple):
        alpha = rng.uniform(w.alpha[0], w.alpha[1], C)
    else:
        alpha = np.full(C, float(w.alpha))
    types = rng.integers(0, max(w.n_types, 1), C)
    genome = float(sum(w.chrom_bins))
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    f32 = torch.float32
    alpha_d = torch.from_numpy(alpha).to(dev, f32)
    totals_d = torch.from_numpy(totals).to(dev, torch.float64)
    types_d = torch.from_numpy(types).to(dev, torch.long)
    out = []
    for ci, nbin in enumerate(w.chrom_bins):
        crng = np.random.default_rng(chrom_ss[ci])
        s = torch.from_numpy(_compartments(crng, w.n_types, nbin)).to(dev, f32)
        ui, ud = _upper_band(nbin, w.band)
        rows, cols = _band_rowmajor(nbin, w.band)
        doff = np.concatenate([[0], np.cumsum([nbin - d for d in range(min(w.band, nbin - 1) + 1)])])
        up_idx = torch.from_numpy(doff[np.abs(cols - rows)] + np.minimum(rows, cols)).to(dev)
        ui_d, ud_d = torch.from_numpy(ui).to(dev), torch.from_numpy(ud).to(dev)
        logd = torch.log(ud_d.to(f32) + 1.0)
        w_sym = torch.where(ud_d > 0, 2.0, 1.0).to(torch.float64)
        P_up = len(ui)
        counts = torch.empty((C, P_up), dtype=torch.int32, device=dev)
        cell_sum = torch.empty(C, dtype=torch.float64, device=dev)
        for c0 in range(0, C, cell_chunk):
            c1 = min(C, c0 + cell_chunk)
            lam = torch.exp(-alpha_d[c0:c1, None] * logd[None, :])
            if w.n_types > 0:
                st = s[types_d[c0:c1]]
                lam *= torch.exp(w.gamma * st[:, ui_d] * st[:, ui_d + ud_d])
            lam *= ((totals_d[c0:c1, None] * nbin / genome) / lam.double().sum(1, keepdim=True)).to(f32)
            cnt = torch.poisson(lam, generator=gen).clamp_(max=65535).to(torch.int32)
            counts[c0:c1] = cnt
            cell_sum[c0:c1] = cnt.double() @ w_sym                 # both triangles
            del lam, cnt
        scale = (nbin / (cell_sum + 1e-15)).to(f32)
        rows_d = torch.from_numpy(rows.astype(np.int32)).to(dev)
        cols_d = torch.from_numpy(cols.astype(np.int32)).to(dev)
        idx_parts, val_parts = [], []
        P_band = len(rows)
        for p0 in range(0, P_band, band_chunk):
            p1 = min(P_band, p0 + band_chunk)
            bandT = counts[:, up_idx[p0:p1]].t().contiguous()      # (positions, cells)
            nz = torch.nonzero(bandT)                               # sorted by (position, cell)
            p, cell = nz[:, 0], nz[:, 1]
            cnt = bandT[p, cell].to(f32)
            val_parts.append(torch.log1p(cnt * scale[cell]))
            idx_parts.append(torch.stack([rows_d[p0 + p], cols_d[p0 + p], cell.to(torch.int32)]))
            del bandT, nz, p, cell, cnt
        del counts
        vals = torch.cat(val_parts) if val_parts else torch.empty(0, dtype=f32, device=dev)
        idx = torch.cat(idx_parts, dim=1) if idx_parts else torch.empty((3, 0), dtype=torch.int32,
                                                                          device=dev)
        del val_parts, idx_parts
        if vals.numel():
            v64 = vals.double()
            m, sd = float(v64.mean()), float(v64.std(unbiased=False))
            del v64
            vals.clamp_(max=m + 15 * sd)
        if pinned:
            from . import _lib
            h_idx = _lib.HostBuffer(max(12 * idx.shape[1], 1), zero=False).array(
                np.int32, (3, idx.shape[1]))
            h_val = _lib.HostBuffer(max(4 * vals.numel(), 1), zero=False).array(
                np.float32, (vals.numel(),))
        else:
            h_idx = np.empty((3, idx.shape[1]), dtype=np.int32)
            h_val = np.empty(vals.numel(), dtype=np.float32)
        torch.from_numpy(h_idx).copy_(idx)
        torch.from_numpy(h_val).copy_(vals)
        del idx, vals
        out.append((h_idx, h_val, (nbin, nbin, C)))
    torch.cuda.empty_cache()
    return out, dict(totals=totals, alpha=alpha, types=types)
