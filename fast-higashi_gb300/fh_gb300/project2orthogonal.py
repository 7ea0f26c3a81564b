"""project2orthogonal on the GPU (drop-in for fasthigashi.project2orthogonal).

Returns (U Vh, S) of matrix (..., d1, d2) as the reference's thin SVD would
(project2orthogonal.py:6-34): the orthonormal polar factor and the singular values in
descending order.  Batches of small tall matrices (d1 <= 320, d2 <= 64) take the
Householder-QR + scaled-Newton kernel; a single tall matrix with d2 <= 64 (the
meta-embedding case) takes the fp64-Gram route.  Wide matrices are transposed.
"""
from __future__ import annotations

from . import _lib


def _polar_tall(M):
    import torch
    batch, n, r = M.shape
    U = torch.empty_like(M)
    st = torch.zeros(1, dtype=torch.int32, device=M.device)
    if n <= 320 and r <= 64:
        _lib.call("fh_polar_f32", _lib.ptr(M), batch, n, r, _lib.ptr(U), None, _lib.ptr(st),
                  _lib.stream_ptr())
    elif r <= 64:
        rp = 16 if r <= 16 else (32 if r <= 32 else 64)
        ws = torch.empty(_lib.value("fh_meta_polar_workspace", n, r), dtype=torch.uint8,
                         device=M.device)
        ssum = torch.zeros(1, dtype=torch.float64, device=M.device)
        for b in range(batch):
            Sp = torch.zeros((n, rp), dtype=torch.float32, device=M.device)
            Sp[:, :r] = M[b]
            Ep = torch.empty_like(Sp)
            _lib.call("fh_meta_polar", _lib.ptr(Sp), n, r, rp, _lib.ptr(Ep), _lib.ptr(ssum),
                      _lib.ptr(ws), ws.numel(), _lib.ptr(st), _lib.stream_ptr())
            U[b] = Ep[:, :r]
    else:
        raise _lib.FHError("project2orthogonal", 2, "more than 64 columns")
    S = torch.empty((batch, r), dtype=torch.float32, device=M.device)
    _lib.call("fh_polar_svals_f32", _lib.ptr(M), _lib.ptr(U), batch, n, r, _lib.ptr(S),
              _lib.stream_ptr())
    return U, S


def project2orthogonal(matrix, rank, compute_device=None):
    import torch
    if not matrix.is_cuda:
        raise _lib.FHError("project2orthogonal", 2, "matrix must be a CUDA tensor")
    d1, d2 = matrix.shape[-2], matrix.shape[-1]
    full = min(d1, d2)
    if rank is None:
        rank = full
    if rank != full:
        raise NotImplementedError("rank below min(matrix.shape[-2:]) is not supported")
    lead = matrix.shape[:-2]
    M = matrix.reshape((-1, d1, d2)).to(torch.float32)
    wide = d1 < d2
    if wide:
        M = M.transpose(-1, -2)
    U, S = _polar_tall(M.contiguous())
    if wide:
        U = U.transpose(-1, -2)
    U = U.reshape(lead + (d1, d2))
    S = S.reshape(lead + (full,))
    if compute_device is not None:
        U = U.to(compute_device)
    return U, S
