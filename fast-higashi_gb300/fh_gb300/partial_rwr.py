"""partial_rwr on the GPU (drop-in for fasthigashi.partial_rwr.partial_rwr).

x is a (cells, b, n) CUDA tensor (the transpose=True tile of Chrom_Dataset.fetch).  The
library's kernel builds P from the tile (partial_rwr.py:84-111) and returns Q_e x with
Q_{t+1} = 0.5 Q_t P + 0.5 I (:112-138).  With force_rwr_epochs < 0 the epoch count follows
the auto-stop rule (:99-126): the first epoch e where max over cells of ||Q_e - Q_{e+1}||_F
< 0.01 stops the walk after Q_{e+1}; n_iter = e (60 and Q_60 when it never stops).
do_conv=True smooths the tile first with the 3 x 3 mean of :79-83 (fh_conv_dense_f32).
do_col=True (with do_rwr) returns Q' (x / bin_cov) instead, Q' the symmetrised, clipped,
row-normalised Q (:131-138, fh_rwr_col_dense); bin_cov is the (cells, n) coverage slice the
reference passes (anything that broadcasts to it).  As in the reference, the output is
transposed only when do_conv or do_rwr is set.
"""
from __future__ import annotations

from . import _lib


def _auto_epochs(x, s0, rows, width):
    import torch
    C = x.shape[0]
    for cap in (12, 60):
        d = torch.empty((C, cap), dtype=torch.float32, device=x.device)
        _lib.call("fh_rwr_dense_deltas", _lib.ptr(x), C, rows, width, s0, cap, _lib.ptr(d),
                  None, _lib.stream_ptr())
        below = (d.max(dim=0).values < 0.01).nonzero()
        if below.numel():
            e = int(below[0, 0].item())
            return e, e + 1
    return 60, 60


def partial_rwr(x, slice_start, slice_end, do_conv, do_rwr, do_col, bin_cov=None, bin_cov_row=None,
                return_rwr_iter=False, force_rwr_epochs=-1, final_transpose=True,
                slice_arrange=False, slice_arrange_size=100, **kw):
    import torch
    n_iter = 0
    if not (do_conv or do_rwr):
        return (x, n_iter) if return_rwr_iter else (x, 0)
    if not (x.is_cuda and x.dtype == torch.float32 and x.dim() == 3):
        raise _lib.FHError("partial_rwr", 1, "x must be a (cells, b, n) float32 CUDA tensor")
    x = x.contiguous()
    if do_conv and x.shape[1] > 1:
        out = torch.empty_like(x)
        _lib.call("fh_conv_dense_f32", _lib.ptr(x), x.shape[0], x.shape[1], x.shape[2],
                  _lib.ptr(out), _lib.stream_ptr())
        x = out
    if do_rwr:
        C, rows, width = x.shape
        if slice_end - slice_start != rows:
            raise _lib.FHError("partial_rwr", 1, "slice must span the tile's rows")
        if force_rwr_epochs < 0:
            n_iter, epochs = _auto_epochs(x, slice_start, rows, width)
        else:
            n_iter = epochs = int(force_rwr_epochs)
        out = torch.empty_like(x)
        if do_col:
            if bin_cov is None:
                raise _lib.FHError("partial_rwr", 1, "do_col needs bin_cov")
            cov = torch.as_tensor(bin_cov).to(x.device, torch.float32)
            cov = cov.expand(C, width).contiguous()
            _lib.call("fh_rwr_col_dense", _lib.ptr(x), C, rows, width, slice_start, epochs,
                      _lib.ptr(cov), _lib.ptr(out), None, _lib.stream_ptr())
        else:
            _lib.call("fh_rwr_dense_f32", _lib.ptr(x), C, rows, width, slice_start, epochs,
                      _lib.ptr(out), None, _lib.stream_ptr())
        x = out
    if final_transpose:
        x = x.permute(1, 2, 0)
    return (x, n_iter) if return_rwr_iter else (x, 0)
