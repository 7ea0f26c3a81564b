"""CPU restatement of the Fast-Higashi fit hot path (TEST INFRASTRUCTURE: the checker).

This module is the oracle.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import it; the product (``fh_gb300``) never does.
It restates, in NumPy, the reference algorithm step by step with the same loop
structure and operation order, in a selectable precision (float64 by default,
float32 to time the reference's arithmetic on host cores).

Parity pin: ``tests/golden/make_golden.py`` runs the reference itself in this
container on seeded inputs and stores its outputs; ``tests/test_oracle_golden.py``
checks this restatement against them.

Reference files (paths within ma-compbio/Fast-Higashi):
  fasthigashi/sparse_for_schic.py      tiling (Chrom_Dataset) and densify
  fasthigashi/partial_rwr.py           partial random walk with restart
  fasthigashi/project2orthogonal.py    polar factor U Vh (thin SVD)
  fasthigashi/parafac_integrative.py   CP-ALS inner solver
  fasthigashi/parafac2_intergrative.py the PARAFAC2-like ALS driver
  fasthigashi/FastHigashi_Wrapper.py   input packing, embedding post-processing
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


# ----------------------------------------------------------------------------------------
# Tiling: restates Chrom_Dataset.__init__ (sparse_for_schic.py:357-510), compact=True.
# ----------------------------------------------------------------------------------------
@dataclass
class BinBatch:
    start: int          # first global row bin
    rows: int           # b
    local: slice        # columns of the compact tile that hold the same bins as the rows
    col: slice          # global column bins of the compact tile
    width: int          # n
    shift: int          # local col = global col - shift


def tile_layout(num_bin: int, bs_bin: int, flank: int):
    """Bin batches of a chromosome in the compact layout (sparse_for_schic.py:401-492)."""
    out = []
    for i in range(0, num_bin, bs_bin):
        b = min(bs_bin, num_bin - i)
        right = flank if num_bin - i - b - flank > 0 else num_bin - i - b
        if i > flank:
            local = slice(flank, flank + b)
            col = slice(i - flank, i + b + right)
            shift = i - flank
            width = b + flank + right
        else:
            local = slice(i, i + b)
            col = slice(0, i + b + right)
            shift = 0
            width = i + b + right
        out.append(BinBatch(i, b, local, col, width, shift))
    return out


def cell_batches(num_cell: int, bs_cell: int):
    return [slice(c, min(c + bs_cell, num_cell)) for c in range(0, num_cell, bs_cell)]


def tile_coo(indices, values, bb: BinBatch, cells: slice):
    """Entries of one (bin batch, cell batch) tile, in tile-local coordinates."""
    r, c, k = indices
    m = (r >= bb.start) & (r < bb.start + bb.rows) & (k >= cells.start) & (k < cells.stop)
    return r[m] - bb.start, c[m] - bb.shift, k[m] - cells.start, values[m]


def densify(rows, cols, cells, vals, b, n, ncell, dtype=np.float64):
    """densify_jit with transpose=True, do_conv=False (sparse_for_schic.py:279-320):
    scatter into a (cells, b+2, n+2) tile at +1 offsets, crop the padding, floor at 1e-8.
    Entries that land in the padding ring are dropped, as the crop drops them."""
    d = np.zeros((ncell, b + 2, n + 2), dtype=dtype)
    d[cells, rows + 1, cols + 1] = vals
    return np.maximum(d[:, 1:-1, 1:-1], dtype(1e-8)).astype(dtype)


# ----------------------------------------------------------------------------------------
# Input packing: restates FastHigashi.pack_training_data_one_process
# (FastHigashi_Wrapper.py:221-366) for one chromosome without a blacklist or batch ids,
# fac_size 1 and a symmetric map, with preprocessing.py:114-193, 474-489.
# ----------------------------------------------------------------------------------------
def pack_chromosome(cells, nbin, reorder, off_diag, merge=1):
    """cells[c] = (row, col, value) of cell c's raw contact matrix (nbin x nbin, canonical CSR
    order).  Returns (indices int32[3, nnz] = (row, col, cell), values float32[nnz], shape)
    as the packed Sparse input of the fit: cells taken in `reorder`, bins merged by `merge`
    (:255-261), contacts beyond `off_diag` dropped (:264-268), bins with no contact in any
    cell removed and renumbered (filter_bin), each cell scaled to total `bins` (normalize_by_
    coverage), then log1p and a clip at mean + 15 std over the chromosome (:358-364)."""
    nb = int(math.ceil(nbin / merge))
    mats = []
    for c in reorder:
        row, col, val = cells[c]
        if merge > 1:
            # the reference divides the coordinates of a canonical COO in place, so its
            # sum_duplicates() call is a no-op: merged duplicates stay separate entries
            row, col = row // merge, col // merge
        keep = np.abs(col - row) <= off_diag
        mats.append((row[keep], col[keep], val[keep].astype(np.float32)))
    # valid bins: any contact in any cell (the bulk's row sums, filter_bin; the reference's
    # buffered x[row, col] += data counts a duplicated coordinate once, which cannot change
    # which rows are positive)
    bulk = np.zeros((nb, nb))
    for row, col, val in mats:
        bulk[row, col] += val
    valid = (bulk / len(mats)).sum(1) > 0
    new_id = np.cumsum(valid) - 1
    new_id[~valid] = -1
    idx, vals = [], []
    for k, (row, col, val) in enumerate(mats):
        n = val.sum()
        val = val * (nb / (n + 1e-15))                    # normalize_by_coverage, scale = bins
        r, c = new_id[row], new_id[col]
        ok = (r != -1) & (c != -1)
        idx.append(np.stack([r[ok], c[ok], np.full(int(ok.sum()), k)]))
        vals.append(val[ok])
    indices = np.concatenate(idx, axis=1).astype(np.int32)
    values = np.log1p(np.concatenate(vals).astype(np.float32))
    values = np.clip(values, None, np.mean(values) + 15 * np.std(values))
    return indices, values, (int(valid.sum()), int(valid.sum()), len(mats))


# ----------------------------------------------------------------------------------------
# Partial RWR: restates partial_rwr.py:75-175.
# ----------------------------------------------------------------------------------------
def rwr_transition(A, s0, s1):
    """P of partial_rwr.py:84-111 for a (C, b, n) tile."""
    dt = A.dtype.type
    b = A.shape[1]
    ar = np.arange(b)
    S2 = np.matmul(A, A.transpose(0, 2, 1))                       # :85
    S2[:, ar, ar] = 0                                             # :86-87
    S1 = A[:, :, s0:s1].copy()                                    # :88
    S2 = (S2 / (S2.sum(1, keepdims=True) + dt(1e-15))) * dt(0.25)  # :90
    S1 = (S1 / (S1.sum(1, keepdims=True) + dt(1e-15))) * dt(0.75)  # :91
    L = S1 + S2                                                   # :93
    L[:, ar, ar] += (L.sum(1) == 0)                               # :96-97
    return L / (L.sum(1, keepdims=True) + dt(1e-15))              # :111


def conv3x3_mean(x):
    """partial_rwr.py:79-83: F.avg_pool2d(x, 3, stride 1, padding 1, ceil_mode=True) on each
    (b, n) tile (zero padding counted, so every output is a sum of nine over 9), then the
    1e-8 floor.  Applied only when b > 1 (:80)."""
    dt = x.dtype.type
    C, b, n = x.shape
    if b <= 1:
        return x
    p = np.zeros((C, b + 2, n + 2), dtype=x.dtype)
    p[:, 1:-1, 1:-1] = x
    s = np.zeros_like(x)
    for di in range(3):
        for dj in range(3):
            s = s + p[:, di:di + b, dj:dj + n]
    return np.maximum(s / dt(9), dt(1e-8))


def partial_rwr(x, slice_start, slice_end, do_rwr=True, do_col=False, bin_cov=None,
                force_rwr_epochs=-1, final_transpose=True, return_rwr_iter=False, do_conv=False):
    """x: (C, b, n).  Returns ((b, n, C) if final_transpose else (C, b, n), n_iter)."""
    n_iter = 0
    if do_conv:
        x = conv3x3_mean(x)
    if do_rwr:
        dt = x.dtype.type
        A = x
        P = rwr_transition(A, slice_start, slice_end)
        b = P.shape[1]
        eye = np.eye(b, dtype=x.dtype)
        Q = np.broadcast_to(eye, P.shape).copy()
        auto = force_rwr_epochs < 0
        epochs = 60 if auto else force_rwr_epochs
        count = 0
        for _ in range(epochs):                                   # :115-126
            Qn = dt(0.5) * np.matmul(Q, P)
            Qn[:, np.arange(b), np.arange(b)] += dt(0.5)
            if auto:
                delta = np.sqrt(((Q - Qn) ** 2).sum(axis=(1, 2)))
                Q = Qn
                if np.max(delta) < 0.01:
                    break
            else:
                Q = Qn
            count += 1
        n_iter = count
        if do_col:                                                # :131-135
            Q = (Q + Q.transpose(0, 2, 1)) * dt(0.5)
            Q = np.maximum(Q, 0)
            Q = Q / (Q.sum(2, keepdims=True) + dt(1e-15))
            A = A / bin_cov[:, None, :]
        x = np.matmul(Q, A)                                       # :138
    if final_transpose and (do_conv or do_rwr):                   # :168-169
        x = x.transpose(1, 2, 0)
    return (x, n_iter) if return_rwr_iter else (x, 0)


# ----------------------------------------------------------------------------------------
# Polar factor: project2orthogonal.py:6-34 (thin SVD, U[:, :rank] Vh[:rank]).
# ----------------------------------------------------------------------------------------
def project2orthogonal(matrix, rank=None):
    U, S, Vh = np.linalg.svd(matrix, full_matrices=False)
    if rank is None:
        rank = min(matrix.shape[-2:])
    return U[..., :rank] @ Vh[..., :rank, :], S[..., :rank]


# ----------------------------------------------------------------------------------------
# CP-ALS: parafac_integrative.py:12-112.
# ----------------------------------------------------------------------------------------
def balance_norm(factors):
    """parafac_integrative.py:19-27: unit columns, the product of norms folded into the last."""
    norm = 1
    for f in factors:
        norm = norm * np.linalg.norm(f, axis=0)
    even = norm + 1e-15
    for i in range(len(factors)):
        factors[i] = factors[i] / (np.linalg.norm(factors[i], axis=0) + 1e-15)
    factors[-1] = factors[-1] * even


def parafac(X, rank, n_iter_max=100, init=None, dtype=np.float64):
    """Returns (factors, loss_norm, loss_x) as parafac_integrative.py:28-112."""
    X = np.asarray(X, dtype=dtype)
    factors = [np.array(f, dtype=dtype) for f in init]
    subs = "ijk"
    balance_norm(factors)
    history = []
    for _ in range(n_iter_max):
        for i in range(3):
            A = np.ones((rank, rank), dtype=dtype)
            for j, f in enumerate(factors):
                if j != i:
                    A = A * (f.T @ f)                             # calc_A :43-48
            others = [j for j in range(3) if j != i]
            spec = "ijk," + ",".join(subs[j] + "r" for j in others) + "->" + subs[i] + "r"
            B = np.einsum(spec, X, *[factors[j] for j in others], optimize=True)   # calc_B :55-62
            A = A + np.eye(rank, dtype=dtype) * dtype(1e-10)      # update_factor :12-15
            factors[i] = np.linalg.solve(A, B.T).T
        Xhat = np.einsum("ir,jr,kr->ijk", *factors, optimize=True)
        loss_recon = float(np.sum((X - Xhat) ** 2))
        loss_norm = float(np.sum(Xhat ** 2))
        loss_x = float(np.sum(Xhat * X))
        history.append((loss_recon, loss_norm, loss_x))
        wdiff = np.nan if len(history) < 2 else (history[-2][0] - history[-1][0]) / history[-2][0]
        if wdiff < 1e-5:
            break
        balance_norm(factors)
    return factors, history[-1][1], history[-1][2]


# ----------------------------------------------------------------------------------------
# The ALS driver: parafac2_intergrative.py:304-740 with an injected initialisation.
# ----------------------------------------------------------------------------------------
@dataclass
class ChromData:
    name: str
    indices: np.ndarray       # int32[3, nnz] (row, col, cell)
    values: np.ndarray        # float32[nnz]
    num_bin: int
    num_cell: int             # good-QC cells: [0, num_cell)
    bs_bin: int
    bs_cell: int
    flank: int
    total_cell: int = 0       # all cells (0: num_cell); cells past num_cell are bad-QC

    def layout(self):
        return tile_layout(self.num_bin, self.bs_bin, self.flank)

    def cells(self):
        return cell_batches(self.num_cell, self.bs_cell)

    def bad_cells(self):
        """Bad-QC cell batches in global cell numbers (sparse_for_schic.py:422-427)."""
        total = max(self.total_cell, self.num_cell)
        return [slice(c, min(c + self.bs_cell, total)) for c in range(self.num_cell, total, self.bs_cell)]

    def tile(self, bb, cs, dtype):
        r, c, k, v = tile_coo(self.indices, self.values, bb, cs)
        return densify(r, c, k, v.astype(dtype), bb.rows, bb.width, cs.stop - cs.start, dtype)


def chrom2size(datas, rank, size_ratio, resolution):
    """parafac2_intergrative.py:558-567."""
    out = {}
    for d in datas:
        s = min(int(d.num_bin * size_ratio * resolution / 1000000), rank)
        out[d.name] = min(out.get(d.name, s), s)
    return out


class ALSOracle:
    """Holds the factor state (A per chromosome dataset, B and D per chromosome, E) and runs
    ALS iterations exactly as Fast_Higashi_core.fit does after init_params."""

    def __init__(self, datas, rank, A_list, B_dict, D_dict, E, n_i, dtype=np.float64, cache_rwr=True,
                 do_conv=False, do_col=False, bin_cov_list=None, bad_bin_cov_list=None,
                 do_rwr=True):
        self.do_conv = do_conv
        self.do_rwr = do_rwr
        self.do_col = do_col
        if do_col:
            if bin_cov_list is None:
                raise ValueError("do_col needs the coverage rows (bin_cov_list)")
            self.bin_cov = [np.asarray(c, dtype=dtype) for c in bin_cov_list]
            self.bad_bin_cov = [None if c is None or np.isscalar(c) else np.asarray(c, dtype=dtype)
                                for c in (bad_bin_cov_list or [None] * len(datas))]
        self.datas = datas
        self.rank = rank
        self.dt = dtype
        self.A_list = [np.array(a, dtype=dtype) for a in A_list]
        self.B = {k: np.array(v, dtype=dtype) for k, v in B_dict.items()}
        self.D = {k: np.array(v, dtype=dtype) for k, v in D_dict.items()}
        self.E = np.array(E, dtype=dtype)
        self.n_i = [int(v) for v in n_i]
        self.size = {d.name: self.B[d.name].shape[0] for d in datas}
        self._cache = {} if cache_rwr else None
        self.rec_errors, self.rec_errors_total = [], []
        self.norm_tensor = None
        self.core_norm = self._core_norm()

    def rwr_tile(self, ci, bi, cj, bad=False):
        """X of one tile after partial RWR with force_rwr_epochs = n_i, as (b, n, C); bad
        selects the bad-QC cell batches (transform, parafac2_intergrative.py:803-827)."""
        key = (ci, bi, cj, bad)
        if self._cache is not None and key in self._cache:
            return self._cache[key]
        d = self.datas[ci]
        bb = d.layout()[bi]
        cs = (d.bad_cells() if bad else d.cells())[cj]
        x = d.tile(bb, cs, self.dt)
        cov = None
        if self.do_col:                                                   # :363, :819
            cov = (self.bad_bin_cov[ci][cs.start - d.num_cell:cs.stop - d.num_cell, bb.col] if bad
                   else self.bin_cov[ci][cs, bb.col])
        out, _ = partial_rwr(x, bb.local.start, bb.local.stop, do_rwr=self.do_rwr,
                             force_rwr_epochs=self.n_i[ci], final_transpose=True,
                             do_conv=self.do_conv, do_col=self.do_col, bin_cov=cov)
        if not (self.do_rwr or self.do_conv):
            # nothing to do: the reference fetches the tile untransposed, (b, n, C) (:345-348)
            out = out.transpose(1, 2, 0)
        out = np.ascontiguousarray(out)
        if self._cache is not None:
            self._cache[key] = out
        return out

    def _core_norm(self):
        """parafac2_intergrative.py:621-632 (per dataset, over bin batches)."""
        out = np.zeros(len(self.datas))
        for ci, d in enumerate(self.datas):
            B, D, A = self.B[d.name], self.D[d.name], self.A_list[ci]
            for i in range(0, d.num_bin, d.bs_bin):
                c = np.einsum("ir,jr,kr->kij", A[i:i + d.bs_bin], B, D, optimize=True)
                out[ci] += float(np.sum(c.astype(np.float64) ** 2)) if self.dt == np.float64 else float(np.sum(c ** 2))
        return out

    def update(self, first_iter=False):
        """update_meta_embedding_interactions (parafac2_intergrative.py:304-540).
        Returns (U per (dataset, bin batch), Y per chromosome, err_x_U, err_x_V, tensor_norm)."""
        dt = self.dt
        E = self.E
        SVD_term = np.zeros((E.shape[1], E.shape[0]), dtype=dt)
        err_x_U = np.zeros(len(self.datas))
        tnorm = np.zeros(len(self.datas))
        U_all = []
        for ci, d in enumerate(self.datas):
            A, B, D = self.A_list[ci], self.B[d.name], self.D[d.name]
            C = E @ D                                                    # :336
            U_list = []
            for bi, bb in enumerate(d.layout()):
                rs = slice(bb.start, bb.start + bb.rows)
                temp = None
                X_last = None
                for cj, cs in enumerate(d.cells()):
                    X = X_last = self.rwr_tile(ci, bi, cj)
                    if first_iter:
                        tnorm[ci] += float(np.sum(X.astype(np.float64) ** 2))   # :369
                    lhs = np.einsum("ir,jr,kr->ikj", A[rs], B, C[cs], optimize=True)   # :374
                    t = np.matmul(X, lhs)                                # :380-383
                    temp = t if temp is None else temp + t
                U, S = project2orthogonal(temp, temp.shape[-1])           # :396
                U = U.astype(dt)
                U_list.append(U)
                err_x_U[ci] += float(np.sum(S))                          # :417
                lhs2 = np.einsum("ir,jr,kr->kij", A[rs], B, D, optimize=True).reshape(D.shape[0], -1)  # :422-423
                ncb = len(d.cells())
                for cj, cs in enumerate(d.cells()):                       # :429-477
                    # the last cell batch of phase 1 is reused, as the reference does (:429)
                    X = X_last if cj == ncb - 1 else self.rwr_tile(ci, bi, cj)
                    proj = np.matmul(U.transpose(0, 2, 1), X)
                    SVD_term[:, cs] += lhs2 @ proj.reshape(-1, proj.shape[-1])
            U_all.append(U_list)
        E_new, _ = project2orthogonal(SVD_term.T, self.rank)              # :483
        E_new = E_new.astype(dt)
        err_x_V = float(np.sum(E_new * SVD_term.T))                       # :486
        Y = {}
        for ci, d in enumerate(self.datas):                               # :488-529
            Yc = np.zeros((d.num_bin, self.size[d.name], self.rank), dtype=dt)
            for bi, bb in enumerate(d.layout()):
                g = 0
                for cj, cs in enumerate(d.cells()):
                    X = self.rwr_tile(ci, bi, cj)
                    g = g + np.einsum("ijk,km,ijl->ilm", X, E_new[cs], U_all[ci][bi], optimize=True)
                Yc[bb.start:bb.start + bb.rows] = g
            Y[ci] = Yc
        self.E = E_new
        return U_all, Y, err_x_U, err_x_V, tnorm

    def iterate(self, iteration, n_iter_parafac=1):
        """One iteration of the fit loop (parafac2_intergrative.py:635-737).  The datasets of a
        chromosome (one per resolution) share its B and D: its CP-ALS runs on their Y stacked
        along the bins, in dataset order, and the A rows go back to each dataset (:674-695)."""
        first = self.norm_tensor is None
        U_all, Y, err_x_U, err_x_V, tnorm = self.update(first_iter=first)
        self.U_last = U_all                      # the projections transform reuses (:750)
        if first:
            self.tensor_norm = tnorm
            self.norm_tensor = np.sqrt(tnorm)
            self.norm_tensor_all = float(np.linalg.norm(self.norm_tensor))
        by_block = self.tensor_norm + self.core_norm - 2 * err_x_U
        rec_V = self.tensor_norm.sum() + self.core_norm.sum() - 2 * err_x_V
        groups = {}
        for ci, d in enumerate(self.datas):                              # :674-695
            groups.setdefault(d.name, []).append(ci)
        for name, ids in groups.items():
            r = self.size[name]
            Yc = np.concatenate([Y[ci] for ci in ids], axis=0)
            Ac = np.concatenate([self.A_list[ci] for ci in ids], axis=0)
            f, _, _ = parafac(Yc, rank=r, n_iter_max=n_iter_parafac,
                              init=[Ac, self.B[name], self.D[name]], dtype=self.dt)
            off = 0
            for ci in ids:
                nb = self.datas[ci].num_bin
                self.A_list[ci] = f[0][off:off + nb]
                off += nb
            self.B[name], self.D[name] = f[1], f[2]
        self.core_norm = self._core_norm()                                # :697-706
        rec = math.sqrt(rec_V) / self.norm_tensor_all                     # :710
        self.rec_errors_total.append(rec)
        self.rec_errors.append(np.sqrt(by_block) / self.norm_tensor)
        return dict(U=U_all, Y=Y, err_x_U=err_x_U, err_x_V=err_x_V, rec_error=rec)

    def fit(self, n_iter_max, n_iter_parafac=1, tol=0.0):
        for it in range(n_iter_max):
            if it % 10 == 0 and it > 0 and n_iter_parafac < 10:          # :636-637
                n_iter_parafac += 1
            self.iterate(it, n_iter_parafac)
            if it >= 1:
                t = self.rec_errors_total
                diff = (self.rec_errors[-2] ** 2 - self.rec_errors[-1] ** 2) / self.rec_errors[-2] ** 2
                tdiff = (t[-2] ** 2 - t[-1] ** 2) / t[-2] ** 2
                if it >= 3 and tol > 0 and (tdiff < tol or diff.max() < tol * 2):
                    break
        return self

    def transform(self, U_all):
        """transform (parafac2_intergrative.py:742-834): final SVD_term over the good and then
        the bad-QC cells with the stored projections and the current factors, then its polar
        factor (total cells x R)."""
        dt = self.dt
        total = max(max(d.total_cell, d.num_cell) for d in self.datas)
        SVD_term = np.zeros((self.E.shape[1], total), dtype=dt)
        for ci, d in enumerate(self.datas):
            A, B, D = self.A_list[ci], self.B[d.name], self.D[d.name]
            for bi, bb in enumerate(d.layout()):
                rs = slice(bb.start, bb.start + bb.rows)
                lhs = np.einsum("ir,jr,kr->kij", A[rs], B, D, optimize=True).reshape(D.shape[0], -1)
                for cj, cs in enumerate(d.cells()):
                    X = self.rwr_tile(ci, bi, cj)
                    proj = np.matmul(U_all[ci][bi].transpose(0, 2, 1), X)
                    SVD_term[:, cs] += lhs @ proj.reshape(-1, proj.shape[-1])
                for cj, cs in enumerate(d.bad_cells()):                      # :803-827
                    X = self.rwr_tile(ci, bi, cj, bad=True)
                    proj = np.matmul(U_all[ci][bi].transpose(0, 2, 1), X)
                    SVD_term[:, cs] += lhs @ proj.reshape(-1, proj.shape[-1])
        E, _ = project2orthogonal(SVD_term.T, self.rank)
        return E


def col_coverage(datas, dtype=np.float64, do_conv=False, mark_inf=True, bad=False):
    """bin_cov of init_params (parafac2_intergrative.py:96-99, 118-142, 266-267), good cells:
    per chromosome, 1e-4 plus, for every (bin batch, cell batch) in loop order, the column
    sums (over the tile's rows) of the auto-stopped do_col=False walk, added at the tile's
    global columns; entries still <= 1e-4 become inf when mark_inf (the do_col feature pass
    of :203-240 runs before that replacement).  bad: bad_bin_cov over the bad-QC cell
    batches instead (:176-200, :268-271)."""
    dt = dtype
    out = []
    for d in datas:
        batches = d.bad_cells() if bad else d.cells()
        c0 = d.num_cell if bad else 0
        n = (max(d.total_cell, d.num_cell) - d.num_cell) if bad else d.num_cell
        cov = np.full((n, d.num_bin), dt(1e-4), dtype=dt)
        for bb in d.layout():
            for cs in batches:
                x = d.tile(bb, cs, dt)
                y, _ = partial_rwr(x, bb.local.start, bb.local.stop, do_rwr=True,
                                   force_rwr_epochs=-1, final_transpose=False, do_conv=do_conv)
                cov[cs.start - c0:cs.stop - c0, bb.col] += y.sum(1)       # :141-142, :199-200
        if mark_inf:
            cov[cov <= dt(1e-4)] = np.inf                                 # :266-267
        out.append(cov)
    return out


# ----------------------------------------------------------------------------------------
# Imputed maps: restates FastHigashi.only_partial_rwr (FastHigashi_Wrapper.py:569-655).
# ----------------------------------------------------------------------------------------
def only_partial_rwr(d, do_conv=False, do_rwr=True, dtype=np.float64):
    """{cell: map} of one chromosome: each (bin batch, cell batch) tile walked with the
    auto-stop (force_rwr_epochs=-1), good batches then bad ones (:576-650), placed at
    [rows, compact columns] (:598-600), then M + M^T with the diagonal halved (:601-605)."""
    out = {}
    for cs in d.cells() + d.bad_cells():
        M = np.zeros((cs.stop - cs.start, d.num_bin, d.num_bin), dtype=dtype)
        for bb in d.layout():
            x = d.tile(bb, cs, dtype)
            y, _ = partial_rwr(x, bb.local.start, bb.local.stop, do_rwr=do_rwr,
                               force_rwr_epochs=-1, final_transpose=False, do_conv=do_conv)
            M[:, bb.start:bb.start + bb.rows, bb.col] = y
        M = M + M.transpose(0, 2, 1)
        for i in range(M.shape[0]):
            m = M[i]
            out[cs.start + i] = m - np.diag(np.diag(m) / 2)
    return out


# ----------------------------------------------------------------------------------------
# Post-processing: restates FastHigashi.fetch_cell_embedding and correct_batch_linear
# (FastHigashi_Wrapper.py:750-878).  The reference calls scikit-learn's TruncatedSVD
# (randomized, unseeded), quantile_transform, LinearRegression and normalize; these are
# restated from their published definitions, with the exact SVD standing for the randomized
# one (they agree when the sketch covers the range, as in the fixtures).
# ----------------------------------------------------------------------------------------
def cell_embedding(E, D_list, dtype=np.float64):
    """Columns of every chromosome's E @ D / ||D||_col, concatenated (:753-758)."""
    E = np.asarray(E, dtype=dtype)
    parts = []
    for D in D_list:
        D = np.asarray(D, dtype=dtype)
        parts.append(E @ (D / np.linalg.norm(D, axis=0, keepdims=True)))
    return np.concatenate(parts, axis=1)


def _interp_last(x, xp, fp):
    """Linear interpolation on increasing xp (ties allowed): for x inside, the segment
    starting at the last xp[j] <= x; outside, the end values."""
    n = len(xp)
    if x < xp[0]:
        return fp[0]
    if x >= xp[n - 1]:
        return fp[n - 1]
    j = int(np.searchsorted(xp, x, side="right")) - 1
    if xp[j] == x:
        return fp[j]
    slope = (fp[j + 1] - fp[j]) / (xp[j + 1] - xp[j])
    return slope * (x - xp[j]) + fp[j]


def quantile_refs(nq):
    """nq evenly spaced probabilities from 0 to 1: t * (1 / (nq - 1)), the last exactly 1."""
    if nq == 1:
        return np.zeros(1)
    step = 1.0 / (nq - 1)
    refs = np.arange(nq, dtype=np.float64) * step
    refs[-1] = 1.0
    return refs


def linear_percentiles(s, refs):
    """Percentiles of sorted s at probabilities refs (given as percentages refs * 100, as
    the reference's caller passes them): virtual index (n - 1) * (p / 100), interpolated
    from the order statistics either side, from the nearer end (a + (b - a) g below
    g = 1/2, b - (b - a)(1 - g) from it)."""
    n = len(s)
    pr = (refs * 100.0) / 100.0
    v = (n - 1) * pr
    v = np.clip(v, 0, n - 1)
    lo = np.floor(v).astype(np.int64)
    hi = np.minimum(lo + 1, n - 1)
    g = v - lo
    a, b = s[lo], s[hi]
    d = b - a
    return np.where(g >= 0.5, b - d * (1 - g), a + d * g)


def quantile_uniform(x, n_quantiles=100):
    """Quantile transform of one column to [0, 1] (the coverage feature, :763): quantiles of
    the values at evenly spaced probabilities (linear interpolation between order
    statistics, made non-decreasing), each value mapped by the mean of the forward
    interpolation and the reversed one (which splits ties evenly), values within 1e-7 of the
    lowest / highest quantile set to 0 / 1."""
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    n = len(x)
    nq = min(n_quantiles, n)
    refs = quantile_refs(nq)
    q = np.maximum.accumulate(linear_percentiles(np.sort(x), refs))
    out = np.empty_like(x)
    for i, v in enumerate(x):
        f = _interp_last(v, q, refs)
        b = _interp_last(-v, -q[::-1], -refs[::-1])
        out[i] = 0.5 * (f - b)
    out[x + 1e-7 > q[-1]] = 1.0
    out[x - 1e-7 < q[0]] = 0.0
    return out


def truncated_svd(Y, k):
    """U_k S_k of Y's top k singular triplets, each component's sign fixed so that its entry
    of largest magnitude (the first such) is positive."""
    Y = np.asarray(Y, dtype=np.float64)
    U, S, Vt = np.linalg.svd(Y, full_matrices=False)
    U, S, Vt = U[:, :k], S[:k], Vt[:k]
    sign = np.sign(Vt[np.arange(k), np.argmax(np.abs(Vt), axis=1)])
    sign[sign == 0] = 1.0
    return U * (S * sign)[None]


def l2_rows(Y):
    """Rows scaled to unit Euclidean norm (zero rows unchanged)."""
    Y = np.asarray(Y, dtype=np.float64)
    n = np.linalg.norm(Y, axis=1, keepdims=True)
    n[n == 0] = 1.0
    return Y / n


def one_hot(labels):
    """Non-float labels as indicator columns of the sorted distinct values (:829-835)."""
    labels = np.asarray(labels)
    uniq = np.unique(labels)
    return (labels[:, None] == uniq[None]).astype(np.float64)


def linear_residual(V, Y, add_intercept_back=False):
    """Y minus its least-squares fit on V with an intercept (:862-866): centred columns, the
    minimum-norm coefficients (pseudo-inverse of the centred V's Gram), the intercept added
    back on request."""
    V = np.asarray(V, dtype=np.float64)
    if V.ndim == 1:
        V = V.reshape((-1, 1))
    Y = np.asarray(Y, dtype=np.float64)
    mv, my = V.mean(0), Y.mean(0)
    Vc, Yc = V - mv, Y - my
    G = Vc.T @ Vc
    w, Q = np.linalg.eigh(G)
    keep = w > 1e-12 * max(w.max(), 1e-300)
    Ginv = (Q[:, keep] / w[keep]) @ Q[:, keep].T
    beta = Ginv @ (Vc.T @ Yc)
    res = Yc - Vc @ beta
    if add_intercept_back:
        res = res + (my - mv @ beta)[None]
    return res


def fetch_cell_embedding(E, D_list, readcount, final_dim, restore_order=False, reorder=None):
    """The store of fetch_cell_embedding (:750-790) with its coverage regression (:785)."""
    emb = cell_embedding(E, D_list)
    cov = quantile_uniform(readcount).reshape((-1, 1))
    embed = truncated_svd(emb, final_dim)
    if restore_order:
        emb = restore_order_rows(emb, reorder)
        embed = restore_order_rows(embed, reorder)
    store = {"embed_all": emb, "embed_raw": embed, "embed_l2_norm": l2_rows(embed),
             "restore_order": restore_order, "coverage_fh": cov}
    correct_batch_linear(store, cov, "coverage_fh", False, reorder)
    return store


def restore_order_rows(x, reorder):
    out = np.zeros_like(x)
    out[np.asarray(reorder)] = x
    return out


def correct_batch_linear(store, var, name, add_intercept_back=False, reorder=None):
    """Regress var out of the stored embedding, then its truncated SVD and row-normalised
    form (:815-878).  var: floats (one column or several) or labels (one-hot)."""
    var = np.asarray(var)
    if store["restore_order"]:
        var = restore_order_rows(var, reorder)
    if var.dtype.kind not in "f":
        var = one_hot(var)
    res = linear_residual(var, store["embed_all"], add_intercept_back)
    red = truncated_svd(res, store["embed_raw"].shape[1])
    store["embed_correct_%s" % name] = red
    store["embed_l2_norm_correct_%s" % name] = l2_rows(red)
    return store


def procrustes_align(X, Y):
    """Rotation Q minimising ||X Q - Y||_F (orthogonal Procrustes); returns X Q."""
    U, _, Vh = np.linalg.svd(X.T @ Y)
    return X @ (U @ Vh)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
