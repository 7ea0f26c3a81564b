"""Imputed contact maps on the GPU: FastHigashi.only_partial_rwr
(fasthigashi/FastHigashi_Wrapper.py:569-655).

For every chromosome and cell the reference runs the partial walk of each bin batch
(do_col=False, auto-stopped per (bin batch, cell batch) call: force_rwr_epochs=-1, good cell
batches then bad ones), places the output at [bin rows, compact columns] of a dense map,
symmetrises it (M + M^T, diagonal halved) and writes it to an HDF5 group per chromosome, a
dataset per raw cell id.  Here the walk runs once over every (tile, cell) with those per-call
epoch counts (the same auto-stop as init_params' coverage pass), and fh_impute_maps builds the
maps of a chunk of cells on the device; a writer receives each map.  h5py is used when it is
importable (the reference's layout); otherwise each chromosome goes to one NumPy file
<chrom>.npy of shape (cells, bins, bins), in raw cell order when a reorder is given.
"""
from __future__ import annotations

import os

import numpy as np

from . import _lib


def _writer_for(out_dir, schic, reorder):
    try:
        import h5py   # noqa: F401
    except ImportError:
        h5py = None
    files = {}

    if h5py is not None:
        f = h5py.File(os.path.join(out_dir, "impute_prwr.hdf5"), "w")

        def write(k, d, cell, m):
            g = files.get(k)
            if g is None:
                g = files[k] = f.create_group(d.chrom)
                g.create_dataset("shape", data=np.asarray([d.num_bin, d.num_bin]))
            g.create_dataset(str(cell), data=m)

        return write, f.close

    def write(k, d, cell, m):
        a = files.get(k)
        if a is None:
            a = files[k] = np.lib.format.open_memmap(
                os.path.join(out_dir, "%s.npy" % d.chrom), mode="w+", dtype=np.float32,
                shape=(d.total_cell_num, d.num_bin, d.num_bin))
        a[cell] = m

    def close():
        for a in files.values():
            a.flush()

    return write, close


def only_partial_rwr(schic, do_conv=False, do_rwr=True, out_dir=None, writer=None,
                     reorder=None, cells_per_chunk=None, device="cuda"):
    """Imputed maps of every cell of every dataset (one per chromosome).  writer(k, dataset,
    cell_id, map) receives each float32 (bins x bins) map, cell_id = reorder[cell] (the raw
    cell id) or the cell's index; without a writer the maps go to out_dir.  Returns the
    per-(tile, cell) walk epochs."""
    import torch
    from .engine import FitEngine
    from .init import auto_epochs
    if writer is None and out_dir is None:
        raise _lib.FHError("only_partial_rwr", 1, "give out_dir or a writer")
    eng = FitEngine(schic, 1, {d.chrom: 1 for d in schic}, None, device, do_rwr=do_rwr,
                    precision="fp32", do_conv=do_conv)
    if do_rwr:
        _, _, cell_ep = auto_epochs(eng, schic, per_cell=True)
    else:
        cell_ep = np.zeros((eng.n_tiles, eng.Ct), dtype=np.int32)
    ep = torch.as_tensor(np.ascontiguousarray(cell_ep, dtype=np.int32)).to(eng.device)
    eng._col_walk(None, ep, to_x=True)        # the plain walk, X in the compact band layout
    close = None
    if writer is None:
        os.makedirs(out_dir, exist_ok=True)
        writer, close = _writer_for(out_dir, schic, reorder)
    P = _lib.ptr
    try:
        for k, d in enumerate(schic):
            nbin = d.num_bin
            per_cell = nbin * nbin * 4
            chunk = cells_per_chunk or max(1, min(eng.Ct, (1 << 30) // per_cell))
            buf = torch.empty((chunk, nbin, nbin), dtype=torch.float32, device=eng.device)
            host = torch.empty((chunk, nbin, nbin), dtype=torch.float32, pin_memory=True)
            for c0 in range(0, eng.Ct, chunk):
                nc = min(chunk, eng.Ct - c0)
                _lib.call("fh_impute_maps", P(eng.tiles_dev), P(eng.row_tile),
                          eng.ds_rows[k].start, nbin, P(eng.X), eng.ldx, c0, nc, P(buf),
                          P(eng.status), eng.sp())
                host[:nc].copy_(buf[:nc], non_blocking=True)
                torch.cuda.current_stream(eng.device).synchronize()
                eng.check_status("only_partial_rwr")
                maps = host[:nc].numpy()
                for i in range(nc):
                    cell = c0 + i
                    writer(k, d, int(reorder[cell]) if reorder is not None else cell, maps[i])
    finally:
        if close is not None:
            close()
    return cell_ep
