"""Embedding post-processing on the GPU: the wrapper's fetch_cell_embedding and
correct_batch_linear (fasthigashi/FastHigashi_Wrapper.py:750-878) over a fitted model's
meta_embedding and D factors.

The reference computes, on the host:
  embed_all   [E D_1 / ||D_1||_col | E D_2 / ||D_2||_col | ...]            (:753-758)
  coverage_fh quantile_transform(read counts, n_quantiles=100)             (:763-764)
  embed_raw   TruncatedSVD(final_dim).fit_transform(embed_all)             (:767-768)
  embed_l2_norm  rows of embed_raw scaled to unit norm                      (:778)
  then correct_batch_linear('coverage_fh'): embed_all minus its least-squares fit on the
  covariate (with an intercept), its TruncatedSVD and row-normalised form    (:815-878)
Here every step runs in libfhgb300.so (csrc/embed.cu).  The truncated SVD is exact: the
embedding is E M (rank <= R), and the regressed one lies in span([E, V, 1]), so its SVD comes
from an fp64 eigen-decomposition in that small span (fh_range_svd) where the reference runs
scikit-learn's randomized sketch, unseeded; the two agree to the sketch's error (the fixtures:
1e-7 to 2e-5).  The component signs follow the reference's rule.  Arrays come back as NumPy
arrays, as the reference's store holds them.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def _dev(device):
    torch = _torch()
    dev = torch.device(device)
    if dev.type != "cuda":
        raise _lib.FHError("postprocess", 2, "the post-processing runs on a CUDA device only")
    return dev


def _f32(x, dev):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.detach().to(dev, torch.float32).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device=dev)


def _f64(x, dev):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.detach().to(dev, torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def cell_embedding(meta_embedding, D_list, device="cuda"):
    """[E D_i / ||D_i||_col for each chromosome i] side by side: float32 (cells x sum r_i)."""
    torch = _torch()
    dev = _dev(device)
    E = _f32(meta_embedding, dev)
    D = torch.cat([_f32(d, dev) for d in D_list], dim=1).contiguous()
    C, R = E.shape
    if D.shape[0] != R:
        raise _lib.FHError("cell_embedding", 1, "every D must have the meta rank's rows")
    m = D.shape[1]
    Y = torch.empty((C, m), dtype=torch.float32, device=dev)
    inv = torch.empty(m, dtype=torch.float32, device=dev)
    P = _lib.ptr
    _lib.call("fh_embed_assemble", P(E), C, R, R, P(D), m, m, P(inv), P(Y), m, _lib.stream_ptr())
    return Y


def quantile_transform_uniform(x, n_quantiles=100, device="cuda"):
    """One column mapped to [0, 1] by its quantiles (float64, length n)."""
    torch = _torch()
    dev = _dev(device)
    xd = _f64(np.asarray(x).reshape(-1) if not isinstance(x, torch.Tensor) else x.reshape(-1),
              dev)
    n = xd.numel()
    out = torch.empty(n, dtype=torch.float64, device=dev)
    ws = torch.empty(max(_lib.value("fh_quantile_workspace", n, n_quantiles), 1),
                     dtype=torch.uint8, device=dev)
    P = _lib.ptr
    _lib.call("fh_quantile_uniform", P(xd), n, n_quantiles, P(out), P(ws), ws.numel(),
              _lib.stream_ptr())
    return out


def linear_residual(V, Y, add_intercept_back=False, device="cuda"):
    """Y minus its least-squares fit on V (cells x p) with an intercept (minimum-norm
    coefficients); the intercept added back on request.  float32 (cells x m)."""
    torch = _torch()
    dev = _dev(device)
    Vd = _f64(V, dev)
    if Vd.dim() == 1:
        Vd = Vd.reshape(-1, 1).contiguous()
    Yf = _f32(Y, dev)
    C, m = Yf.shape
    p = Vd.shape[1]
    out = torch.empty((C, m), dtype=torch.float32, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = torch.empty(_lib.value("fh_lstsq_workspace", p, m), dtype=torch.uint8, device=dev)
    P = _lib.ptr
    _lib.call("fh_lstsq_residual", P(Vd), C, p, P(Yf), m, m, int(bool(add_intercept_back)),
              P(out), m, P(ws), ws.numel(), P(st), _lib.stream_ptr())
    _check(st, "fh_lstsq_residual")
    return out


def truncated_svd_in_span(F, Y, k, device="cuda"):
    """U_k S_k of Y (cells x m) whose columns lie in the column space of F (cells x r):
    (embed float32 cells x k, singular values float64)."""
    torch = _torch()
    dev = _dev(device)
    Ff = _f32(F, dev)
    Yf = _f32(Y, dev)
    C, r = Ff.shape
    m = Yf.shape[1]
    k = int(k)
    if not 0 < k <= min(r, m):
        raise _lib.FHError("truncated_svd", 1, "k must be in [1, min(rank of the span, columns)]")
    out = torch.empty((C, k), dtype=torch.float32, device=dev)
    sig = torch.empty(k, dtype=torch.float64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = torch.empty(_lib.value("fh_range_svd_workspace", r, m, k), dtype=torch.uint8,
                     device=dev)
    P = _lib.ptr
    _lib.call("fh_range_svd", P(Ff), r, C, r, P(Yf), m, m, k, P(out), k, P(sig), P(ws),
              ws.numel(), P(st), _lib.stream_ptr())
    _check(st, "fh_range_svd")
    return out, sig


def l2_normalize(X, device="cuda"):
    """Rows scaled to unit Euclidean norm, zero rows unchanged."""
    torch = _torch()
    dev = _dev(device)
    Xf = _f32(X, dev)
    n, m = Xf.shape
    out = torch.empty_like(Xf)
    P = _lib.ptr
    _lib.call("fh_l2_rows", P(Xf), m, n, m, P(out), m, _lib.stream_ptr())
    return out


def _check(st, what):
    s = int(st.item())
    if s:
        raise _lib.FHError(what, s, "an fp64 eigen-solve did not converge")


def _one_hot(labels):
    """Non-float labels as indicator columns of the sorted distinct values (:829-835)."""
    labels = np.asarray(labels)
    uniq = np.unique(labels)
    return (labels[:, None] == uniq[None]).astype(np.float64)


class EmbeddingPostprocess:
    """fetch_cell_embedding / correct_batch_linear of FastHigashi (FastHigashi_Wrapper.py:
    737-878) over a fit's outputs, in the fit's cell order.

    meta_embedding: cells x R; D_list: each chromosome's D (R x r_i); coverage_feats: the
    read counts (cells x 1, the fit's cell order); label_info: mapping name -> per-cell
    values (the fit's cell order); reorder: the fit's cell order (raw cell of each fitted
    cell), used by restore_order; rank: the default final_dim."""

    def __init__(self, meta_embedding, D_list, coverage_feats, label_info=None, reorder=None,
                 rank=None, device="cuda"):
        self.device = _dev(device)
        self.meta_embedding = meta_embedding
        self.D_list = list(D_list)
        self.coverage_feats = np.asarray(coverage_feats).reshape((-1, 1))
        self.label_info = {} if label_info is None else label_info
        self.reorder = None if reorder is None else np.asarray(reorder)
        self.rank = int(rank if rank is not None else meta_embedding.shape[1])
        self.embedding_storage = None
        self._E = _f32(meta_embedding, self.device)
        self._Y = None

    def restore_order_fun(self, x):
        """Rows put back in the raw cell order (:745-748)."""
        new_x = np.zeros_like(x)
        new_x[self.reorder] = x
        return new_x

    def fetch_cell_embedding(self, final_dim=None, restore_order=False):
        """The store of :750-790: embed_all, embed_raw, embed_l2_norm, restore_order, and the
        coverage-regressed embed_correct_coverage_fh / embed_l2_norm_correct_coverage_fh."""
        final_dim = self.rank if final_dim is None else int(final_dim)
        Y = cell_embedding(self._E, self.D_list, self.device)
        self._Y = Y
        cov = quantile_transform_uniform(self.coverage_feats, 100, self.device)
        self.label_info["coverage_fh"] = cov.cpu().numpy().reshape((-1, 1))
        embed, _ = truncated_svd_in_span(self._E, Y, final_dim, self.device)
        embed_l2 = l2_normalize(embed, self.device)
        store = {"embed_all": Y.cpu().numpy(), "embed_raw": embed.cpu().numpy(),
                 "embed_l2_norm": embed_l2.cpu().numpy(), "restore_order": restore_order}
        if restore_order:
            for key in ("embed_all", "embed_raw", "embed_l2_norm"):
                store[key] = self.restore_order_fun(store[key])
        self.embedding_storage = store
        self.correct_batch_linear("coverage_fh", False)
        return store

    def correct_batch_linear(self, var_to_regress_name, add_intercept_back=False):
        """Regress the named per-cell variable(s) out of embed_all and store the truncated SVD
        of the residual and its row-normalised form (:815-878); labels that are not floats
        are one-hot encoded."""
        if self.embedding_storage is None or self._Y is None:
            raise _lib.FHError("correct_batch_linear", 1, "run fetch_cell_embedding() first")
        names = ([var_to_regress_name] if isinstance(var_to_regress_name, str)
                 else list(var_to_regress_name))
        cols = []
        for name in names:
            v = np.asarray(self.label_info[name])
            if v.dtype.kind != "f":
                v = _one_hot(v)
            cols.append(v.reshape((len(v), -1)).astype(np.float64))
        V = np.concatenate(cols, axis=1)
        label = "_".join(names)
        res = linear_residual(V, self._Y, add_intercept_back, self.device)
        torch = _torch()
        C = V.shape[0]
        F = torch.cat([self._E, _f32(V, self.device),
                       torch.ones((C, 1), dtype=torch.float32, device=self.device)], dim=1)
        k = self.embedding_storage["embed_raw"].shape[-1]
        red, _ = truncated_svd_in_span(F, res, k, self.device)
        red_l2 = l2_normalize(red, self.device)
        red, red_l2 = red.cpu().numpy(), red_l2.cpu().numpy()
        if self.embedding_storage["restore_order"]:
            red, red_l2 = self.restore_order_fun(red), self.restore_order_fun(red_l2)
        self.embedding_storage["embed_correct_%s" % label] = red
        self.embedding_storage["embed_l2_norm_correct_%s" % label] = red_l2
        return self.embedding_storage
