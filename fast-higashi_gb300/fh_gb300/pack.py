"""Input packing on the GPU: raw per-cell contact matrices of one chromosome -> the packed
(row, col, cell) COO the fit reads.

pack_chromosome(cells, nbin, reorder, off_diag, merge=1) does on the device what
FastHigashi.pack_training_data_one_process (fasthigashi/FastHigashi_Wrapper.py:221-366, with
preprocessing.py:114-193, 474-489) does on the host for one chromosome without a blacklist or
batch ids: cells taken in `reorder`, bins merged by `merge`, contacts beyond `off_diag` dropped,
bin rows with no positive contact removed and renumbered, each cell scaled to total the number
of merged bins, log1p, and a clip at mean + 15 std (the kernels: csrc/pack.cu, entry point
fh_pack_chromosome).  Indices agree with the reference's exactly; values to an ulp or two (the
coverage and moment sums run in fp64 where the reference sums fp32).
"""
from __future__ import annotations

import numpy as np

from . import _lib


def pack_chromosome(cells, nbin, reorder, off_diag, merge=1, device="cuda"):
    """cells[c] = (row, col, value) of raw cell c (nbin x nbin, non-negative values).
    Returns (indices int32[3, nnz] = (row, col, cell), values float32[nnz], shape) with the
    arrays as torch tensors on `device`; shape = (kept bins, kept bins, len(reorder))."""
    import torch
    dev = torch.device(device)
    if dev.type != "cuda":
        raise _lib.FHError("pack_chromosome", 2, "the packing runs on a CUDA device only")
    if merge < 1 or off_diag < 0 or nbin <= 0:
        raise _lib.FHError("pack_chromosome", 1, "merge >= 1, off_diag >= 0 and nbin > 0")
    n_raw = len(cells)
    lens = np.array([len(np.asarray(c[2])) for c in cells], dtype=np.int64)
    off = np.zeros(n_raw + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    total = int(off[-1])
    cat = lambda i, dt: (np.concatenate([np.asarray(c[i], dtype=dt) for c in cells])
                         if total else np.zeros(1, dtype=dt))
    row = torch.from_numpy(cat(0, np.int32)).to(dev)
    col = torch.from_numpy(cat(1, np.int32)).to(dev)
    val = torch.from_numpy(cat(2, np.float32)).to(dev)
    off_d = torch.from_numpy(off).to(dev)
    order = torch.from_numpy(np.ascontiguousarray(reorder, dtype=np.int32)).to(dev)
    n_cells = int(order.numel())
    cap = max(total, 1)
    out_idx = torch.empty((3, cap), dtype=torch.int32, device=dev)
    out_val = torch.empty(cap, dtype=torch.float32, device=dev)
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = torch.empty(_lib.value("fh_pack_workspace", n_cells, int(nbin), int(merge), cap),
                     dtype=torch.uint8, device=dev)
    P = _lib.ptr
    _lib.call("fh_pack_chromosome", P(row), P(col), P(val), P(off_d), n_raw, P(order), n_cells,
              int(nbin), int(merge), int(off_diag), P(out_idx), P(out_val), cap, P(counts),
              P(ws), ws.numel(), P(status), _lib.stream_ptr())
    st = int(status.item())
    if st:
        raise _lib.FHError("pack_chromosome", st, "a coordinate or a reorder entry is out of range")
    nnz, kept = (int(v) for v in counts.cpu().tolist())
    return out_idx[:, :nnz], out_val[:nnz], (kept, kept, n_cells)
