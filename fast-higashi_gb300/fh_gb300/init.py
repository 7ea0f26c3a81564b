"""init_params on the GPU (fasthigashi/parafac2_intergrative.py:61-301).

1. A_list = 1 + 0.01 N(0,1) on the host and B = I + 0.01 N (one N(0,1) row added to every
   row of I, as the reference's broadcast does), drawn from torch's generators in the
   reference's order.
2. n_i: the auto-stop rule of partial_rwr.py:99-126 per (bin batch, cell batch), evaluated
   by the library's delta kernel: the batch stops at the first epoch e where
   max_cells ||Q_e - Q_{e+1}||_F < 0.01; n_i[chrom] is the largest stopping epoch
   (:265).  The features use the stopped output Q_{e+1} A as the reference does.
3. Per chromosome, a randomized truncated SVD of the cells x band features (the
   reference's sklearn TruncatedSVD(n_components=r, n_iter=2), :257-258) whose tall
   products F Omega, F^T Q run as the library's X passes; the sketch's orthonormal basis and
   the SVD of F in it come from fh_range_svd (fp64 Gram and Jacobi eigenbasis of the
   (r+10)-column sketch, on the device).  The concatenated features' top-R singular triplets
   give meta_embedding = U[:, :R] and D = (S Vh)[:R] (:283-290): exactly by fh_range_svd when
   they are at most 256 columns wide, else from a randomized range of R + 10 columns (three
   power iterations, each re-orthonormalised) that fh_range_svd resolves; D = E^T [features]
   by the fp64 fh_cross_f32.  Nothing of the factorization runs on the host.
At resolutions finer than 1 Mb the features are pooled to 1 Mb first as the reference pools
them (ll x ll block means of every tile, :102-151), through fh_pool_rows / fh_unpool_rows on the
sketch's products.
With do_col (and do_rwr) the coverage rows bin_cov come first (:96-200): 1e-4 plus the
column sums of the auto-stopped plain walk, every cell batch (good and bad) stopping on its
own; the features are then the do_col walk's output with the same per-batch epochs
(:203-240), and entries <= 1e-4 of the rows become inf (:266-270).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .engine import FitEngine
from .postprocess import truncated_svd_in_span


def _torch():
    import torch
    return torch


def _stop_epochs(deltas, cap, tol=0.01):
    """First epoch e with max over cells of delta[e] < tol, or None if none below cap."""
    m = deltas.max(axis=0)
    below = np.nonzero(m < tol)[0]
    return int(below[0]) if below.size else None


def auto_epochs(eng, schic, per_cell=False):
    """Per-tile stopping epochs and per-dataset n_i (partial_rwr.py:99-126, :265).  With
    per_cell, also the epoch count of every (tile, cell) as the reference's batched loops
    see it: each cell batch, good (:118-142) and bad (:178-200), stops on its own."""
    n_i = np.zeros(len(schic), dtype=np.int64)
    feat_epochs = np.zeros(eng.n_tiles, dtype=np.int32)
    cell_ep = np.zeros((eng.n_tiles, eng.Ct), dtype=np.int32) if per_cell else None
    for cap in (12, 60):
        deltas = eng.auto_deltas(cap, all_cells=per_cell).cpu().numpy()   # (tiles, cells, cap)
        ok = True
        for k, d in enumerate(schic):
            batches = d.cell_slice_list if per_cell else d.cell_slice_list[:d.num_cell_batch]
            for bi in range(d.num_bin_batch):
                t = eng.tile_base[k] + bi
                fe = 0
                for j, cs in enumerate(batches):
                    e = _stop_epochs(deltas[t, cs], cap)
                    if e is None:
                        if cap < 60:
                            ok = False
                            break
                        e, out = 60, 60                   # ran all 60 epochs without stopping
                    else:
                        out = e + 1                       # Q was advanced once more before break
                    if per_cell:
                        cell_ep[t, cs] = out
                    if j < d.num_cell_batch:
                        n_i[k] = max(n_i[k], e)
                        fe = max(fe, out)
                feat_epochs[t] = fe
                if not ok:
                    break
            if not ok:
                break
        if ok:
            return (n_i, feat_epochs, cell_ep) if per_cell else (n_i, feat_epochs)
        n_i[:] = 0
    return (n_i, feat_epochs, cell_ep) if per_cell else (n_i, feat_epochs)


def _chrom_band_rows(eng, ks):
    """Band rows of X holding the datasets ks (one chromosome's resolutions, adjacent)."""
    t = eng.tiles
    x0 = min(int(t["xoff"][eng.tile_base[k]]) for k in ks)
    x1 = 0
    for k in ks:
        last = eng.tile_base[k] + eng.schic[k].num_bin_batch - 1
        x1 = max(x1, int(t["xoff"][last] + t["rows"][last] * t["width"][last]))
    return x0, x1


def randomized_features(eng, ks, n_comp, rng, n_oversamples=10, n_iter=2):
    """U_k S_k (cells x n_comp) of one chromosome's band features F (cells x band rows of its
    datasets ks, every resolution side by side, as the reference concatenates a chromosome's
    features across resolutions).  The sketch's n_comp + n_oversamples columns go through the
    X passes in blocks of at most 128 (the passes' widest operand)."""
    torch = eng.torch
    C = eng.C
    x0, x1 = _chrom_band_rows(eng, ks)
    view = eng.x_rows(x0, x1)                 # (X or the part holding these rows, stride, base)
    X, ld, base = view
    a0 = ((x0 - base) // 128) * 128
    a1 = min(ld, int(math.ceil((x1 - base) / 128) * 128))
    rows = a1 - a0
    n = n_comp + n_oversamples
    dev, f32 = eng.device, torch.float32
    lo, hi = x0 - base - a0, x1 - base - a0
    bufs = {}

    def blocks_of(w):
        return [(c0, min(c0 + 128, w)) for c0 in range(0, w, 128)]

    def buffers(w):
        rp = 128 if w > 64 else (64 if w > 32 else (32 if w > 16 or eng.bf16 else 16))
        if rp not in bufs:
            splits = eng.xg_splits(C, rows)
            bufs[rp] = (torch.zeros((rows, rp), dtype=f32, device=dev),
                        torch.zeros((C, rp), dtype=f32, device=dev),
                        splits, torch.empty((splits, C, rp), dtype=f32, device=dev))
        return rp, bufs[rp]

    def ft_times(Ecells):                     # F^T E: (band rows of k) x n
        out = []
        for c0, c1 in blocks_of(Ecells.shape[1]):
            rp, (W, _, _, _) = buffers(c1 - c0)
            E = torch.zeros((C, rp), dtype=f32, device=dev)
            E[:, :c1 - c0] = Ecells[:, c0:c1]
            eng.x_times_e(a0, rows, C, E, rp, W, view=(X, ld))
            out.append(W[lo:hi, :c1 - c0].clone())
        return torch.cat(out, dim=1)

    def f_times(Qrows):                       # F Q: cells x n
        out = []
        for c0, c1 in blocks_of(Qrows.shape[1]):
            rp, (_, S, splits, part) = buffers(c1 - c0)
            G = torch.zeros((rows, rp), dtype=f32, device=dev)
            G[lo:hi, :c1 - c0] = Qrows[:, c0:c1]
            eng.x_times_g(a0, rows, C, G, rp, splits, part, S, view=(X, ld))
            out.append(S[:, :c1 - c0].clone())
        return torch.cat(out, dim=1)

    # the 1 Mb pooling (:102-151): features of a dataset finer than 1 Mb are its tiles' ll x ll
    # block means; the sketch works in pooled rows through Pm^T (after F^T E) and Pm (before F Q)
    pool = _pooling(eng, ks)
    if pool is not None:
        ft_plain, f_plain = ft_times, f_times
        ft_times = lambda Ecells: pool.pool(ft_plain(Ecells))
        f_times = lambda Qp: f_plain(pool.unpool(Qp))
    omega = torch.from_numpy(rng.standard_normal((C, n)).astype(np.float32)).to(dev)
    # range of F^T (band rows x n), re-orthonormalised after every product (F and F^T alike)
    # so that the power iterations keep the sketch's conditioning at that of F
    Qh = orthonormal_columns(ft_times(omega))
    for _ in range(n_iter):
        Qh = orthonormal_columns(ft_times(orthonormal_columns(f_times(Qh))))
    Bt = f_times(Qh)                          # (Q^T F^T)^T, cells x n
    # F^T = Qh Bt^T  =>  F = Bt Qh^T ; the SVD of Bt (cells x n) gives F's left factors
    k = min(n_comp, Bt.shape[1])
    emb, _ = truncated_svd_in_span(Bt, Bt, k, dev)
    if k < n_comp:
        emb = torch.cat([emb, torch.zeros((C, n_comp - k), dtype=f32, device=dev)], dim=1)
    return emb


class _Pool:
    """The pooling maps of one chromosome's tiles (fh_pool_rows / fh_unpool_rows)."""

    def __init__(self, eng, t0, t1, lls, x0, x1):
        torch = eng.torch
        t = eng.tiles
        pr = [0]
        for k in range(t0, t1):
            ll = lls[k - t0]
            pr.append(pr[-1] + (int(t["rows"][k]) // ll) * (int(t["width"][k]) // ll))
        self.n = t1 - t0
        self.prows = pr[-1]
        self.x0, self.rows = x0, x1 - x0
        self.prow0 = torch.as_tensor(np.asarray(pr, dtype=np.int64)).to(eng.device)
        self.ll = torch.as_tensor(np.asarray(lls, dtype=np.int32)).to(eng.device)
        self.tiles = _lib.ptr(eng.tiles_dev) + t0 * _lib.TILE_DTYPE.itemsize
        self.dev = eng.device
        self.torch = torch

    def pool(self, W):
        W = W.contiguous()
        out = self.torch.empty((self.prows, W.shape[1]), dtype=self.torch.float32,
                               device=self.dev)
        P = _lib.ptr
        _lib.call("fh_pool_rows", self.tiles, self.n, P(self.prow0), P(self.ll), self.x0, P(W),
                  W.shape[1], W.shape[1], P(out), W.shape[1], _lib.stream_ptr())
        return out

    def unpool(self, Qp):
        Qp = Qp.contiguous()
        out = self.torch.empty((self.rows, Qp.shape[1]), dtype=self.torch.float32,
                               device=self.dev)
        P = _lib.ptr
        _lib.call("fh_unpool_rows", self.tiles, self.n, P(self.prow0), P(self.ll), self.x0,
                  self.rows, P(Qp), Qp.shape[1], Qp.shape[1], P(out), Qp.shape[1],
                  _lib.stream_ptr())
        return out


def _pooling(eng, ks):
    """The pooling of datasets ks (one chromosome) when one of them is finer than 1 Mb, else
    None.  ll = ceil(1 Mb / resolution) per dataset (:110)."""
    lls_ds = [int(math.ceil(1000000 / eng.schic[k].resolution)) for k in ks]
    if max(lls_ds) <= 1:
        return None
    t0 = min(eng.tile_base[k] for k in ks)
    t1 = max(eng.tile_base[k] + eng.schic[k].num_bin_batch for k in ks)
    lls = []
    for tt in range(t0, t1):
        k = next(k for k in ks if eng.tile_base[k] <= tt < eng.tile_base[k] + eng.schic[k].num_bin_batch)
        lls.append(max(1, int(math.ceil(1000000 / eng.schic[k].resolution))))
    x0, x1 = _chrom_band_rows(eng, ks)
    return _Pool(eng, t0, t1, lls, x0, x1)


def orthonormal_columns(Q, rel=1e-7):
    """An orthonormal basis of Q's columns (rows x n, n <= 256) on the device: Q's exact SVD in
    its own span (fh_range_svd) as U S, then U; directions below rel of the largest singular
    value (fp32 noise) are dropped."""
    n = Q.shape[1]
    us, sig = truncated_svd_in_span(Q, Q, n, Q.device)
    keep = sig > rel * sig[0]
    m = int(keep.sum().item())
    return (us[:, :m] / sig[:m].float()[None]).contiguous()


def _gemm(A, B):
    """A (n x K) B (K x m) in fp32 on the device (fh_gemm_scale_f32)."""
    torch = _torch()
    A, B = A.contiguous(), B.contiguous()
    out = torch.empty((A.shape[0], B.shape[1]), dtype=torch.float32, device=A.device)
    P = _lib.ptr
    _lib.call("fh_gemm_scale_f32", P(A), A.shape[1], P(B), B.shape[1], None, A.shape[0],
              B.shape[1], A.shape[1], P(out), B.shape[1], _lib.stream_ptr())
    return out


def _cross(A, B):
    """A^T B (A: rows x na, B: rows x nb) summed in fp64 on the device (fh_cross_f32)."""
    torch = _torch()
    A, B = A.contiguous(), B.contiguous()
    out = torch.empty((A.shape[1], B.shape[1]), dtype=torch.float64, device=A.device)
    P = _lib.ptr
    _lib.call("fh_cross_f32", P(A), A.shape[1], A.shape[1], P(B), B.shape[1], B.shape[1],
              A.shape[0], P(out), B.shape[1], _lib.stream_ptr())
    return out


def top_singular(Y, R, rng, n_iter=3, oversample=10):
    """(U_R, S_R) of Y (cells x m) on the device: exact (fh_range_svd in Y's own span) when
    m <= 256, else within a randomized range of R + oversample columns refined by n_iter power
    iterations (each re-orthonormalised)."""
    torch = _torch()
    m = Y.shape[1]
    if m <= 256:
        us, sig = truncated_svd_in_span(Y, Y, R, Y.device)
    else:
        q = min(R + oversample, m, 256)
        omega = torch.from_numpy(rng.standard_normal((m, q)).astype(np.float32)).to(Y.device)
        Z = _gemm(Y, omega)
        for _ in range(n_iter):
            W = orthonormal_columns(_cross(Y, orthonormal_columns(Z)).float())
            Z = _gemm(Y, W)
        F = orthonormal_columns(Z)
        us, sig = truncated_svd_in_span(F, Y, min(R, F.shape[1]), Y.device)
        if us.shape[1] < R:
            pad = R - us.shape[1]
            us = torch.cat([us, torch.zeros((us.shape[0], pad), dtype=us.dtype,
                                            device=us.device)], dim=1)
            sig = torch.cat([sig, torch.zeros(pad, dtype=sig.dtype, device=sig.device)])
    live = sig > 0
    U = torch.where(live[None], us / torch.where(live, sig, torch.ones_like(sig)).float()[None],
                    torch.zeros_like(us))
    return U.contiguous(), sig


def init_params(model, schic, do_conv, do_rwr, do_col, seed=None):
    import torch
    rank = model.rank
    device = model.device
    sizes = model.chrom2size
    A_list = [torch.randn([d.shape[0], sizes[d.chrom]], dtype=torch.float32) * 1e-2 + 1
              for d in schic]
    B_dict = {c: torch.eye(s, device=device).add_(torch.randn(s, device=device), alpha=1e-2)
              for c, s in sizes.items()}
    eng = FitEngine(schic, rank, sizes, None, device, do_rwr=do_rwr,
                    precision=getattr(model, "precision", "fp32"), do_conv=do_conv,
                    do_col=do_col, hbm_budget=getattr(model, "hbm_budget", None))
    model.engine = eng
    if eng.do_col:
        # coverage from the plain walk, then the features from the do_col walk (:96-240)
        n_i, feat_epochs, cell_ep = auto_epochs(eng, schic, per_cell=True)
        eng.compute_coverage(cell_ep)
        eng.col_features(cell_ep)
    elif do_rwr:
        n_i, feat_epochs = auto_epochs(eng, schic)
        eng.set_epochs(feat_epochs)
        eng.run_rwr()
    else:
        n_i = np.zeros(len(schic), dtype=np.int64)
        eng.set_n_i(n_i)
        eng.run_rwr()
    rng = np.random.default_rng(seed)
    feats, cols = [], []
    start = 0
    for ci, name in enumerate(eng.names):
        ks = [k for k in range(len(schic)) if eng.chrom_index[k] == ci]
        f = randomized_features(eng, ks, sizes[name], rng)
        feats.append(f)
        cols.append((name, start, start + f.shape[1]))
        start += f.shape[1]
    Call = torch.cat(feats, dim=1).contiguous()            # cells x sum(r), on the device
    R = min(rank, Call.shape[1])
    U, _ = top_singular(Call, R, rng)
    E = torch.zeros((Call.shape[0], rank), dtype=torch.float32, device=Call.device)
    E[:, :R] = U
    SVh = torch.zeros((rank, Call.shape[1]), dtype=torch.float32, device=Call.device)
    SVh[:R] = _cross(U, Call).float()                       # U^T Call = S Vh
    model.meta_embedding = E.to(device)
    model.D_dict = {c: SVh[:, a:b].contiguous().to(device) for c, a, b in cols}
    model.A_list = A_list
    model.B_dict = B_dict
    model.n_i = np.asarray(n_i)
    if eng.do_col:
        eng.finalize_coverage()
        model.bin_cov_list, model.bad_bin_cov_list = eng.coverage_views()
        eng.cov_src = (model.bin_cov_list, model.bad_bin_cov_list)
    else:
        model.bin_cov_list = [None] * len(schic)
        model.bad_bin_cov_list = [0] * len(schic)
    eng.set_n_i(model.n_i)
    eng.run_rwr()
