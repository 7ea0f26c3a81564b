"""project2orthogonal on the GPU (drop-in for fasthigashi.project2orthogonal).

Returns (U Vh, S) of matrix (..., d1, d2) as the reference's thin SVD would
(project2orthogonal.py:6-34): the orthonormal polar factor and the singular values in
descending order.  Matrices that fit in shared memory take the Householder-QR + Newton
kernel; taller ones with d2 <= 128 (the meta-embedding case) take the fp64-Gram route.  S
comes from a one-sided Jacobi of the symmetric U^T M.  Wide matrices are transposed.
"""
from __future__ import annotations

from . import _lib


def _polar_tall(M):
    import torch
    batch, n, r = M.shape
    U = torch.empty_like(M)
    S = torch.empty((batch, r), dtype=torch.float32, device=M.device)
    st = torch.zeros(1, dtype=torch.int32, device=M.device)
    if r <= 128 and _lib.value("fh_polar_smem", n, r) <= 227 * 1024:
        _lib.call("fh_polar_f32", _lib.ptr(M), batch, n, r, _lib.ptr(U), None, _lib.ptr(st),
                  _lib.stream_ptr())
    elif r <= 128:
        rp = 16 if r <= 16 else (32 if r <= 32 else (64 if r <= 64 else 128))
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
        raise _lib.FHError("project2orthogonal", 2, "more than 128 columns")
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
