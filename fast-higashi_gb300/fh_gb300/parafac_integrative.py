"""CP-ALS on one 3-way tensor (drop-in for fasthigashi.parafac_integrative.parafac).

parafac(X, rank, n_iter_max, init=[A, B, D]) runs n_iter_max sweeps of the library's CP-ALS
kernels (the steps of parafac_integrative.py:28-112 with the normal-equation systems formed
and inverted in fp64, balance_norm, the 1e-5 relative-change stop) and returns (factors, loss_norm, loss_x) with
loss_norm = ||[[A,B,D]]||^2 and loss_x = <[[A,B,D]], X> of the last sweep.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def parafac(X, rank, n_iter_max=100, init=None, verbose=False, common_factor=None):
    import torch
    if init is None or len(init) != 3:
        raise _lib.FHError("parafac", 1, "init=[A, B, D] is required")
    if not torch.cuda.is_available():
        raise _lib.FHError("parafac", 5, "no CUDA device")
    dev = torch.device("cuda")
    X = torch.as_tensor(X).to(dev, torch.float32)
    nbin, r, R = X.shape
    if r != rank:
        raise _lib.FHError("parafac", 1, "X.shape[1] must equal rank")
    rp = 16 if R <= 16 else (32 if R <= 32 else (64 if R <= 64 else 128))
    ld = max(rp, rank)
    if ld > 128 or R > 128:
        raise _lib.FHError("parafac", 2, "ranks above 128 are not supported")
    A = torch.zeros((nbin, ld), dtype=torch.float32, device=dev)
    B = torch.zeros((1, ld, ld), dtype=torch.float32, device=dev)
    D = torch.zeros((1, rp, ld), dtype=torch.float32, device=dev)
    Y = torch.zeros((nbin, ld, rp), dtype=torch.float32, device=dev)
    A[:, :rank] = torch.as_tensor(init[0]).to(dev, torch.float32)
    B[0, :rank, :rank] = torch.as_tensor(init[1]).to(dev, torch.float32)
    D[0, :R, :rank] = torch.as_tensor(init[2]).to(dev, torch.float32)
    Y[:, :rank, :R] = X
    k_row0 = list(range(0, nbin, 8))
    meta = np.array([0, nbin, rank, 0, len(k_row0)] + [0] * len(k_row0) + k_row0 +
                    [min(8, nbin - r0) for r0 in k_row0], dtype=np.int32)
    meta_d = torch.from_numpy(meta).to(dev)
    ws = torch.empty(_lib.value("fh_cp_workspace", 1, len(k_row0), ld, rp), dtype=torch.uint8,
                     device=dev)
    core = torch.zeros(1, dtype=torch.float64, device=dev)
    cross = torch.zeros(1, dtype=torch.float64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    P = _lib.ptr
    _lib.call("fh_cp_als", 1, len(k_row0), P(meta_d), P(A), P(B), P(D), P(Y), ld, rp, R, ld,
              int(n_iter_max), P(core), P(cross), P(ws), ws.numel(), P(st), _lib.stream_ptr())
    if int(st.item()):
        raise _lib.FHError("parafac", int(st.item()))
    factors = [A[:, :rank].contiguous(), B[0, :rank, :rank].contiguous(), D[0, :R, :rank].contiguous()]
    return factors, float(core.item()), float(cross.item())
