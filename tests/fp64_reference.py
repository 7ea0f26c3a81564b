"""FP64 restatement of the fit on a torch device (TEST INFRASTRUCTURE: the precision yardstick).

The fit loop of the reference (fasthigashi/partial_rwr.py:75-138, project2orthogonal.py:6-34,
parafac2_intergrative.py:304-737, parafac_integrative.py:12-112) with every array a torch
float64 tensor, so a full-size fit (10,000 cells at 500 kb) runs on a GPU in minutes instead of
hours on host cores.  It is exact-arithmetic equal to the reference; the rounding it leaves is
fp64's.  Three choices make it fast, none of which changes the exact result:
  * cells are not split into batches (the reference's cell batching only orders sums);
  * each iteration makes two passes over the RWR output X per bin batch instead of three:
    W = X^T E gives temp_i = W_i M_i (M_i = D diag(A_i) B^T, the reference's lhs contracted
    with E) and, with the new E, the projected tensor Y_i = U_i^T W_i; S^T = X G^T with
    G_i = U_i M_i^T gives SVD_term (the reference's lhs2 @ U^T X);
  * the per-bin polar factors are batched on the device: Householder QR of temp_i, then the
    polar factor of the r x r triangle by Newton's iteration with Higham's scaling (a matrix
    that does not converge falls back to a host SVD); the sum of singular values is
    trace(U^T temp).
It does not import the oracle (so benchmark code may use it as a checker); tests/
test_precision.py pins it against the numpy oracle (oracle/fh_oracle.py) first.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

F64 = torch.float64


@dataclass
class BinBatch:
    start: int
    rows: int
    local: slice      # the batch's rows inside its compact columns
    col: slice        # compact columns in chromosome bins
    width: int
    shift: int        # first compact column


def tile_layout(num_bin, bs_bin, flank):
    """Bin batches of a chromosome in the compact layout (sparse_for_schic.py:401-492): rows
    [i, i + b), columns from i - flank (clipped at 0) to i + b + flank (clipped at num_bin)."""
    out = []
    for i in range(0, num_bin, bs_bin):
        b = min(bs_bin, num_bin - i)
        right = flank if num_bin - i - b - flank > 0 else num_bin - i - b
        if i > flank:
            out.append(BinBatch(i, b, slice(flank, flank + b), slice(i - flank, i + b + right),
                                b + flank + right, i - flank))
        else:
            out.append(BinBatch(i, b, slice(i, i + b), slice(0, i + b + right), i + b + right, 0))
    return out


@dataclass
class ChromRecord:
    """One chromosome's COO (row, col, cell) and its batching."""
    name: str
    indices: np.ndarray
    values: np.ndarray
    num_bin: int
    num_cell: int
    bs_bin: int
    bs_cell: int
    flank: int

    def layout(self):
        return tile_layout(self.num_bin, self.bs_bin, self.flank)


def polar(m):
    """The polar factor U (U Vh of the thin SVD, project2orthogonal.py:6-34) of every matrix of
    a (batch, n, r) float64 stack with n >= r, and the sum of all their singular values."""
    Q, Rt = torch.linalg.qr(m)
    r = Rt.shape[-1]
    X = Rt.clone()
    eye = torch.eye(r, dtype=F64, device=m.device)
    for _ in range(40):
        Xi = torch.linalg.inv(X)
        nx = torch.linalg.norm(X, dim=(1, 2))
        ni = torch.linalg.norm(Xi, dim=(1, 2))
        z = torch.sqrt(ni / nx)[:, None, None]
        Xn = 0.5 * (z * X + Xi.transpose(1, 2) / z)
        d = torch.linalg.norm(Xn - X, dim=(1, 2)) / torch.linalg.norm(Xn, dim=(1, 2))
        X = Xn
        if bool((d < 1e-14).all()):
            break
    ortho = torch.linalg.norm(X.transpose(1, 2) @ X - eye, dim=(1, 2))
    bad = ~torch.isfinite(ortho) | (ortho > 1e-10)
    if bool(bad.any()):
        idx = torch.nonzero(bad).flatten()
        Uh, _, Vh = np.linalg.svd(m[idx].cpu().numpy(), full_matrices=False)
        Up = torch.from_numpy(Uh @ Vh).to(m.device)
    U = Q @ X
    if bool(bad.any()):
        U[idx] = Up
    ssum = float((U * m).sum())
    return U, ssum


def polar_single(m):
    """Polar factor and singular values of one (C, R) matrix (the meta polar, :483-486)."""
    U, S, Vh = torch.linalg.svd(m, full_matrices=False)
    return U @ Vh, S


def transition(A, s0, s1):
    """The column-stochastic P of partial_rwr.py:84-111 (do_conv=False) for a (cells, b, n)
    float64 tile."""
    b = A.shape[1]
    ar = torch.arange(b, device=A.device)
    S2 = A @ A.transpose(1, 2)
    S2[:, ar, ar] = 0
    S1 = A[:, :, s0:s1]
    S2 = (S2 / (S2.sum(1, keepdim=True) + 1e-15)) * 0.25
    S1 = (S1 / (S1.sum(1, keepdim=True) + 1e-15)) * 0.75
    L = S1 + S2
    L[:, ar, ar] += (L.sum(1) == 0).to(F64)
    return L / (L.sum(1, keepdim=True) + 1e-15)


def rwr_tile(A, s0, s1, epochs, rp=0.5):
    """partial_rwr.py:84-138 (do_conv=False, do_col=False, force_rwr_epochs=epochs) on a
    (cells, b, n) float64 tile: Q_{t+1} = rp Q_t P + (1 - rp) I from Q_0 = I (:109,116-118;
    rp may be a tensor that requires grad); returns Q_epochs A."""
    b = A.shape[1]
    P = transition(A, s0, s1)
    eye = torch.eye(b, dtype=F64, device=A.device)
    Q = eye.expand_as(P).clone()
    for _ in range(epochs):
        Q = rp * (Q @ P) + (1 - rp) * eye
    return Q @ A


def dense_tiles(datas, C, device, cell_chunk=2048):
    """(dataset index, bin batch index, layout, floored dense tile (C, b, n) float64) for every
    bin batch: densify_jit's +1 padding ring, crop and 1e-8 floor (sparse_for_schic.py:
    279-320) from the oracle's ChromData records."""
    dev = torch.device(device)
    for ci, d in enumerate(datas):
        r, c, k = (torch.as_tensor(np.asarray(v, dtype=np.int64)).to(dev) for v in d.indices)
        v = torch.as_tensor(np.asarray(d.values)).to(dev).to(F64)
        for bi, bb in enumerate(d.layout()):
            m = (r >= bb.start) & (r < bb.start + bb.rows)
            rr, cc, kk, vv = r[m] - bb.start, c[m] - bb.shift, k[m], v[m]
            keep = (cc >= -1) & (cc <= bb.width)          # the +1 padding ring
            rr, cc, kk, vv = rr[keep], cc[keep], kk[keep], vv[keep]
            out = torch.empty((C, bb.rows, bb.width), dtype=F64, device=dev)
            for c0 in range(0, C, cell_chunk):
                c1 = min(C, c0 + cell_chunk)
                sel = (kk >= c0) & (kk < c1)
                dense = torch.zeros((c1 - c0, bb.rows + 2, bb.width + 2), dtype=F64, device=dev)
                dense[kk[sel] - c0, rr[sel] + 1, cc[sel] + 1] = vv[sel]
                out[c0:c1] = torch.clamp(dense[:, 1:-1, 1:-1], min=1e-8)
            yield ci, bi, bb, out


def balance_norm(f):
    norm = 1
    for x in f:
        norm = norm * torch.linalg.norm(x, dim=0)
    even = norm + 1e-15
    f = [x / (torch.linalg.norm(x, dim=0) + 1e-15) for x in f]
    f[-1] = f[-1] * even
    return f


def parafac(Y, rank, n_iter_max, init):
    """parafac_integrative.py:28-112 (loss history, 1e-5 relative stop, balance_norm)."""
    f = balance_norm([x.clone() for x in init])
    eye = torch.eye(rank, dtype=F64, device=Y.device)
    specs = ["ijk,jr,kr->ir", "ijk,ir,kr->jr", "ijk,ir,jr->kr"]
    hist = []
    for _ in range(n_iter_max):
        for i in range(3):
            G = torch.ones((rank, rank), dtype=F64, device=Y.device)
            others = [j for j in range(3) if j != i]
            for j in others:
                G = G * (f[j].T @ f[j])
            B = torch.einsum(specs[i], Y, *[f[j] for j in others])
            f[i] = torch.linalg.solve(G + eye * 1e-10, B.T).T
        Xhat = torch.einsum("ir,jr,kr->ijk", *f)
        hist.append(float(((Y - Xhat) ** 2).sum()))
        wdiff = float("nan") if len(hist) < 2 else (hist[-2] - hist[-1]) / hist[-2]
        if wdiff < 1e-5:
            break
        f = balance_norm(f)
    return f


class FP64Fit:
    """Factor state and cached RWR tiles; ``fit(n)`` runs n iterations of the fit loop."""

    def __init__(self, datas, rank, A_list, B_dict, D_dict, E, n_i, device, cell_chunk=2048):
        dev = torch.device(device)
        self.dev = dev
        self.datas = datas
        self.rank = rank
        t = lambda x: torch.as_tensor(np.asarray(x), dtype=F64).to(dev)
        self.A = [t(a) for a in A_list]
        self.B = {k: t(v) for k, v in B_dict.items()}
        self.D = {k: t(v) for k, v in D_dict.items()}
        self.E = t(E)
        self.C = self.E.shape[0]
        self.size = {d.name: self.B[d.name].shape[0] for d in datas}
        self.X = {}
        self.tnorm = np.zeros(len(datas))
        for ci, bi, bb, A in dense_tiles(datas, self.C, dev, cell_chunk):
            out = rwr_tile(A, bb.local.start, bb.local.stop, int(n_i[ci]))
            self.X[(ci, bi)] = out
            self.tnorm[ci] += float((out ** 2).sum())
        self.norm_tensor = np.sqrt(self.tnorm)
        self.norm_all = float(np.linalg.norm(self.norm_tensor))
        self.core = self._core_norm()
        self.W = {}           # X^T E per bin batch for the current E (the next iteration's temp)
        self.rec_errors_total = []

    def _core_norm(self):
        out = np.zeros(len(self.datas))
        for ci, d in enumerate(self.datas):
            B, D, A = self.B[d.name], self.D[d.name], self.A[ci]
            for i in range(0, d.num_bin, d.bs_bin):
                c = torch.einsum("ir,jr,kr->kij", A[i:i + d.bs_bin], B, D)
                out[ci] += float((c ** 2).sum())
        return out

    def iterate(self, n_iter_parafac):
        E = self.E
        R = self.rank
        SVD = torch.zeros((self.C, E.shape[1]), dtype=F64, device=self.dev)    # SVD_term^T
        err_u = np.zeros(len(self.datas))
        U_all = {}
        for ci, d in enumerate(self.datas):
            A, B, D = self.A[ci], self.B[d.name], self.D[d.name]
            for bi, bb in enumerate(d.layout()):
                rs = slice(bb.start, bb.start + bb.rows)
                X = self.X[(ci, bi)].reshape(self.C, -1)                   # (C, b n)
                W = self.W.get((ci, bi))
                if W is None:
                    W = (X.T @ E).reshape(bb.rows, bb.width, -1)           # (b, n, R)
                M = torch.einsum("mr,ir,jr->imj", D, A[rs], B)             # (b, R, r)
                temp = torch.bmm(W, M)                                     # (b, n, r)
                U, ssum = polar(temp)
                U_all[(ci, bi)] = U
                err_u[ci] += ssum
                Gt = torch.bmm(U, M.transpose(1, 2)).reshape(-1, E.shape[1])   # (b n, R)
                SVD += X @ Gt
        E_new, _ = polar_single(SVD)
        err_v = float((E_new * SVD).sum())
        for ci, d in enumerate(self.datas):
            Yc = torch.zeros((d.num_bin, self.size[d.name], R), dtype=F64, device=self.dev)
            for bi, bb in enumerate(d.layout()):
                X = self.X[(ci, bi)].reshape(self.C, -1)
                W = (X.T @ E_new).reshape(bb.rows, bb.width, -1)          # (b, n, R)
                self.W[(ci, bi)] = W
                Yc[bb.start:bb.start + bb.rows] = torch.bmm(U_all[(ci, bi)].transpose(1, 2), W)
            r = self.size[d.name]
            f = parafac(Yc, r, n_iter_parafac, [self.A[ci], self.B[d.name], self.D[d.name]])
            self.A[ci], self.B[d.name], self.D[d.name] = f
        self.E = E_new
        rec_v = self.tnorm.sum() + self.core.sum() - 2 * err_v
        self.core = self._core_norm()
        self.rec_errors_total.append(math.sqrt(rec_v) / self.norm_all)

    def fit(self, n_iter_max, n_iter_parafac=1):
        for it in range(n_iter_max):
            if it % 10 == 0 and it > 0 and n_iter_parafac < 10:
                n_iter_parafac += 1
            self.iterate(n_iter_parafac)
        return self


def chrom_datas(coo, names, bs_bins, bs_cells, flank):
    """ChromRecords from COO triples (indices, values, shape)."""
    out = []
    for (idx, val, shape), name, bsb, bsc in zip(coo, names, bs_bins, bs_cells):
        out.append(ChromRecord(name, idx, val, int(shape[0]), int(shape[2]), int(bsb), int(bsc),
                               int(flank)))
    return out


def cell_embedding(E, D_list):
    """The user-facing cell embedding before its final TruncatedSVD (FastHigashi_Wrapper.py:
    750-761): E times each chromosome's D with unit columns, concatenated (cells x sum r)."""
    E = np.asarray(E, dtype=np.float64)
    parts = []
    for D in D_list:
        D = np.asarray(D, dtype=np.float64)
        parts.append(E @ (D / np.linalg.norm(D, axis=0, keepdims=True)))
    return np.concatenate(parts, axis=1)


def gram_error(F, F_ref):
    """||F F^T - G G^T||_F / ||G G^T||_F (cell-cell similarities; invariant to any rotation
    of the embedding's columns), from the small Gram products only."""
    F = np.asarray(F, dtype=np.float64)
    G = np.asarray(F_ref, dtype=np.float64)
    a = np.linalg.norm(F.T @ F) ** 2
    b = np.linalg.norm(G.T @ G) ** 2
    c = np.linalg.norm(F.T @ G) ** 2
    return float(math.sqrt(max(a + b - 2 * c, 0.0)) / math.sqrt(b))


def aligned_error(E, E_ref):
    """Relative Frobenius error of E after the orthogonal Procrustes rotation onto E_ref."""
    E = np.asarray(E, dtype=np.float64)
    E_ref = np.asarray(E_ref, dtype=np.float64)
    U, _, Vh = np.linalg.svd(E.T @ E_ref)
    return float(np.linalg.norm(E @ (U @ Vh) - E_ref) / max(np.linalg.norm(E_ref), 1e-300))
