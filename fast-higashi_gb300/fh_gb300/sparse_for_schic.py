"""Sparse per-cell contact container and bin-batch tiling (drop-in for fasthigashi.sparse_for_schic).

``Sparse`` is the host COO container of one chromosome (row bin, column bin, cell), with the
reference's row-bin CSR index and slicing (fasthigashi/sparse_for_schic.py:58-275).
``Chrom_Dataset`` computes the reference's bin-batch / cell-batch tiling in the compact band
layout (sparse_for_schic.py:356-510) and keeps the contacts on the GPU: the COO is uploaded
once and sorted into per-(bin batch, cell) segments by the library's contact-build kernels;
``fetch`` densifies a tile on the device (sparse_for_schic.py:588-613).
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import _lib


def calc_offset(dims):
    """Row-major strides of a shape (sparse_for_schic.py:15-18)."""
    dims = np.asarray(dims)
    off = np.ones_like(dims)
    off[:-1] = np.cumprod(dims[:0:-1])[::-1]
    return off


def unfold(indices, shape):
    """Flat index of a multi-index array (sparse_for_schic.py:28-36)."""
    shape = np.asarray(shape)
    flat = calc_offset(shape).astype(np.int64) @ np.asarray(indices, dtype=np.int64)
    assert (flat >= 0).all() and (flat < np.prod(shape.astype(np.int64))).all()
    return flat


def fold(flat, shape):
    """Inverse of unfold (sparse_for_schic.py:39-54)."""
    off = calc_offset(shape).astype(np.int64)
    out = np.empty((len(shape), len(flat)), dtype=np.int64)
    rem = np.asarray(flat, dtype=np.int64)
    for i in range(len(shape) - 1):
        out[i], rem = np.divmod(rem, off[i])
    out[-1] = rem
    return out


class Sparse:
    """COO tensor with a CSR index over dim 0 (sparse_for_schic.py:58-275)."""

    def __init__(self, indices, values, shape, indptr=None, copy=True, verbose=False):
        self.ndim = len(shape)
        self.indices = np.array(indices, copy=True) if copy else np.asarray(indices)
        self.values = np.array(values, copy=True) if copy else np.asarray(values)
        self.shape = np.array(shape, dtype=np.int64)
        self.indptr = None if indptr is None else np.array(indptr)
        self.verbose = verbose
        assert self.indices.shape == (self.ndim, len(self.values))
        assert (self.indices >= 0).all()
        assert (self.indices < self.shape[:, None]).all()

    def sort_indices(self, dim=0, force=False):
        """Orders entries by dim 0 (stable) and builds indptr (sparse_for_schic.py:133-182)."""
        assert dim == 0
        if not force and self.indptr is not None:
            return
        row = self.indices[0]
        if len(row) and (np.diff(row) < 0).any():
            order = np.argsort(row, kind="stable")
            self.indices = np.ascontiguousarray(self.indices[:, order])
            self.values = np.ascontiguousarray(self.values[order])
            row = self.indices[0]
        counts = np.bincount(row, minlength=int(self.shape[0]))
        self.indptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)

    def slicing(self, idx, dim=0):
        assert dim == 0 and isinstance(idx, slice) and idx.step in (None, 1)
        ind, val, shape, start = self.get_slice_idx_value(idx)
        ind = ind.copy()
        ind[0] -= start
        return Sparse(ind, val, shape)

    def get_slice_idx_value(self, idx, dim=0, device="cpu"):
        """Indices/values of rows idx (sparse_for_schic.py:200-213); indices are global."""
        assert dim == 0 and isinstance(idx, slice) and idx.step in (None, 1)
        if self.indptr is None:
            self.sort_indices()
        start = idx.start if idx.start is not None else 0
        stop = min(idx.stop if idx.stop is not None else int(self.shape[0]), int(self.shape[0]))
        lo, hi = self.indptr[start], self.indptr[stop]
        return (self.indices[:, lo:hi], self.values[lo:hi],
                (stop - start,) + tuple(int(s) for s in self.shape[1:]), start)

    def indexing(self, idx, dim=0):
        assert dim == 0 and 0 <= idx < self.shape[0]
        if self.indptr is None:
            self.sort_indices()
        lo, hi = self.indptr[idx], self.indptr[idx + 1]
        return Sparse(self.indices[1:, lo:hi], self.values[lo:hi], tuple(self.shape[1:]))

    def __getitem__(self, item):
        if isinstance(item, (int, np.integer)):
            return self.indexing(int(item))
        if isinstance(item, slice):
            return self.slicing(item)
        raise NotImplementedError

    def permute(self, *dims, inplace=False):
        assert tuple(sorted(dims)) == tuple(range(self.ndim))
        dims = np.asarray(dims)
        ind, shape = self.indices[dims], self.shape[dims]
        indptr = self.indptr if dims[0] == 0 else None
        if inplace:
            self.indices, self.shape, self.indptr = ind, shape, indptr
            return self
        return Sparse(ind, self.values, shape, indptr, verbose=self.verbose)

    def reshape(self, *dims, inplace=False):
        dims = np.array(dims, dtype=np.int64)
        total = int(np.prod(self.shape))
        if (dims == -1).any():
            assert (dims == -1).sum() == 1
            dims[dims == -1] = total // -int(np.prod(dims))
        assert int(np.prod(dims)) == total
        ind = fold(unfold(self.indices, self.shape), dims)
        if inplace:
            self.indices, self.shape, self.ndim = ind, dims, len(dims)
            self.indptr = None
            return self
        return Sparse(ind, self.values, dims, verbose=self.verbose)

    def filter_max_distance(self, max_distance=100):
        m = np.abs(self.indices[1] - self.indices[0]) <= max_distance
        self.indices = self.indices[:, m]
        self.values = self.values[m]
        self.indptr = None

    def split(self, bins, dim):
        bins = list(bins)
        edges = [0] + bins + [int(self.shape[dim])]
        chunk = np.digitize(self.indices[dim], bins)
        order = np.argsort(chunk, kind="stable")
        out = []
        for k in range(len(edges) - 1):
            sel = order[chunk[order] == k]
            ind = self.indices[:, sel].copy()
            ind[dim] -= edges[k]
            shape = tuple(self.shape[:dim]) + (edges[k + 1] - edges[k],) + tuple(self.shape[dim + 1:])
            out.append(Sparse(ind, self.values[sel], shape))
        return (o for o in out)

    def to_dense(self):
        v = np.zeros(tuple(int(s) for s in self.shape))
        v[tuple(self.indices)] = self.values
        return v

    def to_scipy(self):
        from scipy.sparse import coo_matrix
        return coo_matrix((self.values, tuple(self.indices)), tuple(int(s) for s in self.shape))

    def to_csr(self):
        from scipy.sparse import csr_matrix
        return csr_matrix((self.values, tuple(self.indices)), tuple(int(s) for s in self.shape))

    def numel(self):
        return int(np.prod(self.shape))

    def __len__(self):
        return int(self.shape[0])


class BinBatch:
    """Slices of one bin batch in the compact layout (sparse_for_schic.py:457-492)."""

    __slots__ = ("start", "rows", "local", "col", "width", "shift")

    def __init__(self, start, rows, local, col, width, shift):
        self.start, self.rows, self.local = start, rows, local
        self.col, self.width, self.shift = col, width, shift


def compact_layout(num_bin, bs_bin, flank):
    """Bin batches of bs_bin rows with columns [i - flank, i + b + flank) clipped to the
    chromosome; compact column = chromosome column - shift (sparse_for_schic.py:457-492)."""
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


class Chrom_Dataset:
    """One chromosome's contacts tiled into bin batches x cell batches
    (sparse_for_schic.py:356-510).  ``compact`` must be True (the band layout the fit
    uses); ``upper_sim`` is not supported (the wrapper passes False)."""

    def __init__(self, tensor, bs_bin, bs_cell, good_qc_num=-1, kind="hic", upper_sim=False,
                 compact=False, flank=0, chrom="chr1", resolution=10000):
        if not isinstance(tensor, Sparse):
            raise TypeError("Chrom_Dataset takes a Sparse tensor")
        if not compact:
            raise NotImplementedError("only the compact band layout is supported")
        if upper_sim:
            raise NotImplementedError("upper_sim=True is not supported")
        if kind != "hic":
            raise NotImplementedError("only kind='hic' is supported")
        tensor.sort_indices()
        self.tensor = tensor
        self.resolution = resolution
        self.chrom = chrom
        self.length = int(tensor.shape[0])
        self.num_bin = int(tensor.shape[0])
        self.total_cell_num = int(tensor.shape[-1])
        self.num_cell = self.total_cell_num if good_qc_num == -1 else int(good_qc_num)
        self.bs_bin = int(bs_bin)
        self.bs_cell = int(bs_cell)
        self.kind = kind
        self.upper_sim = upper_sim
        self.compact = compact
        self.flank = int(flank)
        self.batches = compact_layout(self.num_bin, self.bs_bin, self.flank)
        self.bin_slice_list = [slice(bb.start, bb.start + bb.rows) for bb in self.batches]
        self.local_bin_slice_list = [bb.local for bb in self.batches]
        self.col_bin_slice_list = [bb.col for bb in self.batches]
        good = [slice(c, min(c + self.bs_cell, self.num_cell)) for c in range(0, self.num_cell, self.bs_cell)]
        bad = [slice(c, min(c + self.bs_cell, self.total_cell_num))
               for c in range(self.num_cell, self.total_cell_num, self.bs_cell)]
        self.cell_slice_list = good + bad
        self.num_bin_batch = len(self.batches)
        self.num_cell_batch = len(good)
        self.num_cell_batch_bad = len(bad)
        self.kind_list = [[kind] * len(good) for _ in self.batches]
        self.bad_kind_list = [[kind] * len(bad) for _ in self.batches]
        self.uniq_kind = np.unique(self.kind_list)
        self.shape = [self.num_bin, self.bs_bin + 2 * self.flank, self.num_cell]
        self._store = None

    def __len__(self):
        return self.length

    def pin_memory(self):
        """The contacts live on the GPU once uploaded; nothing to pin."""
        return self

    # ---- device-side contact store (built lazily for fetch; the fit builds its own) ----
    def _device_store(self, device):
        if self._store is None or self._store.device != device:
            self._store = ContactStore([self], device)
        return self._store

    def fetch(self, bin_id, cell_id, save_context, transpose=False, good_qc=True, **kwargs):
        """Dense tile of one (bin batch, cell batch) on the device, floored at 1e-8:
        (cells, b, n) if transpose else (b, n, cells) (sparse_for_schic.py:588-613)."""
        import torch
        device = torch.device(save_context["device"])
        if device.type != "cuda":
            raise _lib.FHError("fetch", 2, "the contact store lives on a CUDA device")
        t0 = time.perf_counter()
        st = self._device_store(device)
        cs = self.cell_slice_list[cell_id if good_qc else self.num_cell_batch + cell_id]
        bb = self.batches[bin_id]
        out = torch.empty((cs.stop - cs.start, bb.rows, bb.width), dtype=torch.float32, device=device)
        _lib.call("fh_densify_tile", _lib.ptr(st.tiles_dev), bin_id, st.n_cells, cs.start,
                  cs.stop - cs.start, _lib.ptr(st.offsets), _lib.ptr(st.entries), _lib.ptr(out),
                  _lib.stream_ptr())
        if not transpose:
            out = out.permute(1, 2, 0)
        return (out, [time.perf_counter() - t0]), self.kind

    def fetch_bad(self, bin_id, cell_id, **kwargs):
        return self.fetch(bin_id, cell_id, good_qc=False, **kwargs)

    def norm(self):
        return float(np.sqrt(np.sum(np.square(self.tensor.values.astype(np.float64)))))


_PINNED = {}


def _pin(arr):
    """Page-locks a host array in place (once per buffer) so that its H2D copy runs as a DMA
    from pinned memory at the link's bandwidth; the registration lasts as long as the array."""
    import weakref
    import torch
    key = (arr.ctypes.data, arr.nbytes)
    if arr.nbytes == 0 or key in _PINNED:
        return arr
    rt = torch.cuda.cudart()
    if int(rt.cudaHostRegister(arr.ctypes.data, arr.nbytes, 0)) != 0:
        return arr                      # stays pageable: the copy still works, only slower
    owner = arr if arr.base is None else arr.base
    _PINNED[key] = weakref.finalize(owner, lambda p=arr.ctypes.data: (
        _PINNED.pop(key, None), rt.cudaHostUnregister(p)))
    return arr


class ContactStore:
    """Packed per-(tile, cell) contact segments of one or more datasets on a CUDA device.

    Built by the library's counting sort: fh_contacts_count -> fh_exclusive_scan ->
    fh_contacts_scatter, one chromosome at a time, from the host COO (H2D once)."""

    def __init__(self, datasets, device, tiles=None, tile_base=None, stream=None):
        import torch
        self.device = device
        self.n_cells = datasets[0].total_cell_num
        if tiles is None:
            tiles, tile_base = tile_table(datasets)
        self.tiles_np = tiles
        self.tiles_dev = torch.from_numpy(tiles.view(np.uint8).copy()).to(device)
        self.n_tiles = len(tiles)
        self.stream = stream
        self.meta = [(d.bs_bin, base, d.num_bin_batch) for d, base in zip(datasets, tile_base)]
        # H2D of the host COO (Sparse.indices int32 x 3, values fp32), once, from page-locked
        # host memory (the arrays are registered in place, no host copy)
        self.coo = []
        host = []                       # keeps every source alive until the copies land
        for d in datasets:
            t = d.tensor
            hi = _pin(np.ascontiguousarray(np.asarray(t.indices, dtype=np.int32)))
            hv = _pin(np.ascontiguousarray(np.asarray(t.values, dtype=np.float32)))
            host += [hi, hv]
            idx = torch.from_numpy(hi).to(device, non_blocking=True)
            val = torch.from_numpy(hv).to(device, non_blocking=True)
            self.coo.append((idx, val, int(val.numel())))
        torch.cuda.current_stream(device).synchronize()
        del host
        self.h2d_bytes = sum(i.numel() * 4 + v.numel() * 4 for i, v, _ in self.coo)
        self.counts = torch.zeros(self.n_tiles * self.n_cells, dtype=torch.int32, device=device)
        self.cursor = torch.zeros_like(self.counts)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.offsets = torch.empty(self.n_tiles * self.n_cells + 1, dtype=torch.int64, device=device)
        ws_bytes = _lib.value("fh_scan_workspace", self.counts.numel())
        self.scan_ws = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
        self.count_and_scan()
        total = int(self.offsets[-1].item())
        self.entries = torch.empty(max(total, 1) * 2, dtype=torch.int32, device=device)
        self.scatter()
        st = int(self.status.item())
        if st:
            raise _lib.FHError("contact build", st)
        self.nnz_packed = total

    def count_and_scan(self):
        sp = _lib.stream_ptr(self.stream)
        self.counts.zero_()
        for (bs_bin, base, nbb), (idx, val, nnz) in zip(self.meta, self.coo):
            _lib.call("fh_contacts_count", _lib.ptr(idx[0]), _lib.ptr(idx[1]), _lib.ptr(idx[2]),
                      nnz, bs_bin, _lib.ptr(self.tiles_dev), base, nbb, self.n_cells,
                      _lib.ptr(self.counts), _lib.ptr(self.status), sp)
        _lib.call("fh_exclusive_scan", _lib.ptr(self.counts), self.counts.numel(),
                  _lib.ptr(self.offsets), _lib.ptr(self.scan_ws), self.scan_ws.numel(), sp)

    def scatter(self):
        sp = _lib.stream_ptr(self.stream)
        self.cursor.zero_()
        for (bs_bin, base, nbb), (idx, val, nnz) in zip(self.meta, self.coo):
            _lib.call("fh_contacts_scatter", _lib.ptr(idx[0]), _lib.ptr(idx[1]), _lib.ptr(idx[2]),
                      _lib.ptr(val), nnz, bs_bin, _lib.ptr(self.tiles_dev), base, nbb,
                      self.n_cells, _lib.ptr(self.offsets), _lib.ptr(self.cursor),
                      _lib.ptr(self.entries), sp)

    def rebuild(self):
        """Re-runs the contact build from the device-resident COO (no host sync)."""
        self.count_and_scan()
        self.scatter()


def tile_table(datasets, chrom_index=None, ranks=None, n_rwr=None, order=None):
    """fh_tile records for the bin batches of the datasets (in the given order), with band
    rows, bin rows and projection offsets laid out consecutively.  Returns (tiles,
    tile_base) where tile_base[k] is the first tile of datasets[k]."""
    order = list(range(len(datasets))) if order is None else order
    recs = []
    base = [0] * len(datasets)
    xoff = brow = uoff = 0
    for k in order:
        d = datasets[k]
        base[k] = len(recs)
        ci = 0 if chrom_index is None else chrom_index[k]
        r = 0 if ranks is None else ranks[k]
        ni = 0 if n_rwr is None else int(n_rwr[k])
        for bb in d.batches:
            recs.append((ci, bb.start, bb.rows, bb.width, bb.shift, bb.local.start, r, ni,
                         xoff, brow, uoff))
            xoff += bb.rows * bb.width
            brow += bb.rows
            uoff += bb.rows * bb.width * r
    tiles = np.array(recs, dtype=_lib.TILE_DTYPE)
    return tiles, base
