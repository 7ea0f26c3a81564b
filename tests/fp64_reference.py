"""FP64 restatement of the fit on a torch device (TEST INFRASTRUCTURE: the precision yardstick).

The algorithm of ``oracle.fh_oracle.ALSOracle`` (which restates the reference step by step and
cites it: fasthigashi/partial_rwr.py:75-138, project2orthogonal.py:6-34,
parafac2_intergrative.py:304-737, parafac_integrative.py:12-112), with every array a torch
float64 tensor, so a full-size fit (10,000 cells at 500 kb) runs on a GPU in minutes instead of
hours on host cores.  Cells are not split into batches: in exact arithmetic the reference's
cell batching only changes summation order.  ``tests/test_precision.py`` pins this module
against the numpy oracle before using it to state the FP64 error of the fp32 and bf16 forms.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from oracle import fh_oracle as O

F64 = torch.float64


def polar(m):
    """U Vh of the thin SVD and S (project2orthogonal.py:6-34), batched over leading dims.
    Batches of small matrices go through LAPACK on the host (a loop of per-matrix device
    SVD calls is far slower for them); single large matrices stay on the device."""
    if m.dim() == 3:
        U, S, Vh = np.linalg.svd(m.detach().cpu().numpy(), full_matrices=False)
        return torch.from_numpy(U @ Vh).to(m.device), torch.from_numpy(S).to(m.device)
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
        SVD = torch.zeros((E.shape[1], self.C), dtype=F64, device=self.dev)
        err_u = np.zeros(len(self.datas))
        U_all = {}
        for ci, d in enumerate(self.datas):
            A, B, D = self.A[ci], self.B[d.name], self.D[d.name]
            Cm = E @ D
            for bi, bb in enumerate(d.layout()):
                rs = slice(bb.start, bb.start + bb.rows)
                X = self.X[(ci, bi)]                                    # (C, b, n)
                lhs = torch.einsum("ir,jr,kr->ikj", A[rs], B, Cm)         # (b, C, r)
                temp = torch.bmm(X.permute(1, 2, 0), lhs)                # (b, n, r)
                U, S = polar(temp)
                U_all[(ci, bi)] = U
                err_u[ci] += float(S.sum())
                lhs2 = torch.einsum("ir,jr,kr->kij", A[rs], B, D).reshape(D.shape[0], -1)
                proj = torch.bmm(U.transpose(1, 2), X.permute(1, 2, 0))  # (b, r, C)
                SVD += lhs2 @ proj.reshape(-1, self.C)
        E_new, _ = polar(SVD.T)
        err_v = float((E_new * SVD.T).sum())
        for ci, d in enumerate(self.datas):
            Yc = torch.zeros((d.num_bin, self.size[d.name], R), dtype=F64, device=self.dev)
            for bi, bb in enumerate(d.layout()):
                X = self.X[(ci, bi)]
                XE = torch.einsum("kij,km->ijm", X, E_new)               # (b, n, R)
                Yc[bb.start:bb.start + bb.rows] = torch.bmm(U_all[(ci, bi)].transpose(1, 2), XE)
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
    """ChromData records of the oracle from COO triples (indices, values, shape)."""
    out = []
    for (idx, val, shape), name, bsb, bsc in zip(coo, names, bs_bins, bs_cells):
        out.append(O.ChromData(name, idx, val, int(shape[0]), int(shape[2]), int(bsb), int(bsc),
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
    return O.rel_err(O.procrustes_align(E, E_ref), E_ref)
