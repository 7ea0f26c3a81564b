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
        """Moves the host COO into page-locked memory (exact-size cudaHostAlloc buffers, as the
        reference pins its tiles' host copies), so every host-to-device copy of the contacts
        runs at the link's bandwidth; the arrays keep their values and layout."""
        t = self.tensor
        if not (_lib.host_pinned(t.indices.ctypes.data, t.indices.nbytes) and
                _lib.host_pinned(t.values.ctypes.data, t.values.nbytes)):
            t.indices = _lib.pinned_copy(np.asarray(t.indices, dtype=np.int32))
            t.values = _lib.pinned_copy(np.asarray(t.values, dtype=np.float32))
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
    if arr.nbytes == 0 or key in _PINNED or _lib.host_pinned(arr.ctypes.data, arr.nbytes):
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
    fh_contacts_scatter, dataset by dataset in tile order, from the host COO.  The H2D copies
    run on their own stream from page-locked host memory, one event per dataset, so a caller
    that builds dataset k (build(k)) and starts work on it while dataset k + 1 is still in
    flight overlaps the copies with its own kernels; each dataset's offsets are scanned on their
    own and chained onto the previous dataset's total on the device (fh_scan_add_base), and the
    segment buffer is sized by its bound (one slot per contact), so nothing waits on the host
    until finish()."""

    def __init__(self, datasets, device, tiles=None, tile_base=None, stream=None, order=None,
                 defer=False):
        import torch
        self.torch = torch
        self.device = device
        self.n_cells = datasets[0].total_cell_num
        if tiles is None:
            tiles, tile_base = tile_table(datasets, order=order)
        self.tiles_np = tiles
        self.tiles_dev = torch.from_numpy(tiles.view(np.uint8).copy()).to(device)
        self.n_tiles = len(tiles)
        self.stream = stream
        self.meta = [(d.bs_bin, base, d.num_bin_batch) for d, base in zip(datasets, tile_base)]
        self.order = list(range(len(datasets))) if order is None else list(order)
        # H2D of the host COO (Sparse.indices int32 x 3, values fp32) on a copy stream, from
        # page-locked host memory (the arrays are registered in place, no host copy)
        main = self._main()
        self.copy_stream = torch.cuda.Stream(device=device)
        self.copy_stream.wait_stream(main)
        self.coo = [None] * len(datasets)
        self.ready = [None] * len(datasets)
        self._host = []                 # keeps every source alive until the copies land
        with torch.cuda.stream(self.copy_stream):
            for k in self.order:
                t = datasets[k].tensor
                hi = _pin(np.ascontiguousarray(np.asarray(t.indices, dtype=np.int32)))
                hv = _pin(np.ascontiguousarray(np.asarray(t.values, dtype=np.float32)))
                self._host += [hi, hv]
                idx = torch.from_numpy(hi).to(device, non_blocking=True)
                val = torch.from_numpy(hv).to(device, non_blocking=True)
                self.coo[k] = (idx, val, int(val.numel()))
                ev = torch.cuda.Event()
                ev.record(self.copy_stream)
                self.ready[k] = ev
        self.h2d_bytes = sum(i.numel() * 4 + v.numel() * 4 for i, v, _ in self.coo)
        C = self.n_cells
        self.counts = torch.zeros(self.n_tiles * C, dtype=torch.int32, device=device)
        self.cursor = torch.zeros_like(self.counts)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.offsets = torch.zeros(self.n_tiles * C + 1, dtype=torch.int64, device=device)
        self.bases = torch.zeros(len(datasets) + 1, dtype=torch.int64, device=device)
        n_max = max(nbb for _, _, nbb in self.meta) * C
        self.scan_ws = torch.empty(_lib.value("fh_scan_workspace", n_max), dtype=torch.uint8,
                                   device=device)
        bound = sum(nnz for _, _, nnz in self.coo)
        self.entries = torch.empty(max(bound, 1) * 2, dtype=torch.int32, device=device)
        self.nnz_packed = None
        if not defer:
            self.build_all()
            self.finish()

    def _main(self):
        torch = self.torch
        return self.stream if self.stream is not None else torch.cuda.current_stream(self.device)

    def build(self, k):
        """Counts, offsets and segments of dataset k on the caller's stream, after its copy."""
        main = self._main()
        with self.torch.cuda.stream(main):
            self._build(k, main)

    def _build(self, k, main):
        main.wait_event(self.ready[k])
        sp = main.cuda_stream
        P = _lib.ptr
        bs_bin, base, nbb = self.meta[k]
        idx, val, nnz = self.coo[k]
        C = self.n_cells
        start, n = base * C, nbb * C
        self.counts[start:start + n].zero_()
        self.cursor[start:start + n].zero_()
        _lib.call("fh_contacts_count", P(idx[0]), P(idx[1]), P(idx[2]), nnz, bs_bin,
                  P(self.tiles_dev), base, nbb, C, P(self.counts), P(self.status), sp)
        # the datasets before this one (in tile order) end at offsets[start]: keep that total,
        # scan this dataset's counts from zero, then add it back
        self.bases[k:k + 1].copy_(self.offsets[start:start + 1])
        _lib.call("fh_exclusive_scan", P(self.counts[start:]), n, P(self.offsets[start:]),
                  P(self.scan_ws), self.scan_ws.numel(), sp)
        _lib.call("fh_scan_add_base", P(self.offsets[start:]), n + 1, P(self.bases[k:]), sp)
        _lib.call("fh_contacts_scatter", P(idx[0]), P(idx[1]), P(idx[2]), P(val), nnz, bs_bin,
                  P(self.tiles_dev), base, nbb, C, P(self.offsets), P(self.cursor),
                  P(self.entries), sp)

    def build_all(self):
        main = self._main()
        with self.torch.cuda.stream(main):
            self.offsets[:1].zero_()
        for k in self.order:
            self.build(k)

    def finish(self):
        """Waits for the build, checks its status and releases the host sources."""
        self._main().synchronize()
        self.copy_stream.synchronize()
        self._host = []
        st = int(self.status.item())
        if st:
            raise _lib.FHError("contact build", st)
        self.nnz_packed = int(self.offsets[-1].item())

    def rebuild(self):
        """Re-runs the contact build from the device-resident COO (no host sync)."""
        self.build_all()


def coo_chunks(nnz, buf_bytes, n_arrays, align=256):
    """The chunks of a budgeted contact build: (buffer half, byte offset of each array's slot
    in that half, first contact, contacts) for nnz contacts whose n_arrays arrays (4 bytes per
    contact each) pass through two halves of a buffer of buf_bytes, alternately.  Every slot
    starts on a 256-byte boundary and a chunk holds a multiple of 64 contacts (the last one
    the rest)."""
    half = (buf_bytes // 2) // align * align
    m_max = (half // (4 * n_arrays)) // 64 * 64
    if nnz > 0 and m_max <= 0:
        raise _lib.FHError("contact build", 1, "no room for a chunk of the COO")
    slots = [a * m_max * 4 for a in range(n_arrays)]
    return [(j & 1, [j % 2 * half + s for s in slots], e0, min(m_max, nnz - e0))
            for j, e0 in enumerate(range(0, nnz, m_max))] if nnz > 0 else []


class StreamedContacts:
    """The contact build for a fit whose device memory is budgeted: one dataset at a time.

    The host COO stays where the caller holds it (page-locked in place).  build(k) passes over
    dataset k's contacts twice in chunks, each chunk copied by the copy engine into one of two
    buffers the caller lends (double-buffered on a copy stream, so the copy of chunk j + 1 runs
    under the kernel on chunk j): fh_contacts_count on the (row, column, cell) chunks, the scan
    of the counts, then fh_contacts_scatter on the full chunks (12 + 16 bytes per contact over
    the host link).  The (tile, cell) segments go to the buffer the caller names, with offsets
    local to the dataset (its tiles counted from its first), so the walk of dataset k runs right
    after it and the next build reuses the same memory."""

    CHUNK_ALIGN = 256

    def __init__(self, datasets, device, tiles, tile_base, status, order=None):
        import torch
        self.torch = torch
        self.device = device
        self.n_cells = datasets[0].total_cell_num
        self.tiles_np = tiles
        self.tiles_dev = torch.from_numpy(tiles.view(np.uint8).copy()).to(device)
        self.n_tiles = len(tiles)
        self.meta = [(d.bs_bin, base, d.num_bin_batch) for d, base in zip(datasets, tile_base)]
        self.order = list(range(len(datasets))) if order is None else list(order)
        self.status = status
        self.src = [None] * len(datasets)
        for k in self.order:
            t = datasets[k].tensor
            hi = _pin(np.ascontiguousarray(np.asarray(t.indices, dtype=np.int32)))
            hv = _pin(np.ascontiguousarray(np.asarray(t.values, dtype=np.float32)))
            self.src[k] = (hi, hv, int(hv.size))
        self.nnz = [s[2] for s in self.src]
        self.link_bytes = 0                 # host -> device bytes copied so far
        C = self.n_cells
        n_max = max(nbb for _, _, nbb in self.meta) * C
        self.counts = torch.zeros(n_max, dtype=torch.int32, device=device)
        self.cursor = torch.zeros_like(self.counts)
        self.offsets = torch.zeros(n_max + 1, dtype=torch.int64, device=device)
        self.scan_ws = torch.empty(_lib.value("fh_scan_workspace", n_max), dtype=torch.uint8,
                                   device=device)
        self.copy = torch.cuda.Stream(device=device)

    def entries_bytes(self, k):
        return 8 * self.nnz[k]

    def _chunked(self, k, buf_ptr, buf_bytes, arrays, kernel, stream):
        """kernel(device pointers of the chunk's arrays, m) over dataset k's contacts in chunks,
        each chunk's arrays (row, col, cell[, val]: 4 bytes per contact each) copied into one
        half of [buf_ptr, buf_ptr + buf_bytes)."""
        torch = self.torch
        hi, hv, nnz = self.src[k]
        srcs = [hi[0], hi[1], hi[2], hv][:len(arrays)]
        free = [None, None]
        for b, offs, e0, m in coo_chunks(nnz, buf_bytes, len(arrays), self.CHUNK_ALIGN):
            if free[b] is not None:
                self.copy.wait_event(free[b])
            else:
                ev = torch.cuda.Event()
                ev.record(stream)           # after what the stream issued before this build
                self.copy.wait_event(ev)
            dst = []
            for off, src in zip(offs, srcs):
                d = buf_ptr + off
                _lib.call("fh_memcpy_async", d, src.ctypes.data + e0 * 4, m * 4,
                          self.copy.cuda_stream)
                dst.append(d)
            self.link_bytes += m * 4 * len(srcs)
            ready = torch.cuda.Event()
            ready.record(self.copy)
            stream.wait_event(ready)
            kernel(dst, m)
            done = torch.cuda.Event()
            done.record(stream)
            free[b] = done

    def build(self, k, entries_ptr, stream, buf_ptr, buf_bytes):
        """Segments of dataset k into entries_ptr (entries_bytes(k) bytes), offsets into
        self.offsets[:num_bin_batch * cells + 1], on the given torch stream; the COO chunks
        pass through [buf_ptr, buf_ptr + buf_bytes) (device memory not used meanwhile)."""
        P = _lib.ptr
        bs_bin, base, nbb = self.meta[k]
        C = self.n_cells
        n = nbb * C
        sp = stream.cuda_stream
        tiles = P(self.tiles_dev) + base * _lib.TILE_DTYPE.itemsize
        with self.torch.cuda.stream(stream):
            self.counts[:n].zero_()
            self.cursor[:n].zero_()
        if self.nnz[k]:
            self._chunked(k, buf_ptr, buf_bytes, "rcl", lambda d, m: _lib.call(
                "fh_contacts_count", d[0], d[1], d[2], m, bs_bin, tiles, 0, nbb, C,
                P(self.counts), P(self.status), sp), stream)
        _lib.call("fh_exclusive_scan", P(self.counts), n, P(self.offsets), P(self.scan_ws),
                  self.scan_ws.numel(), sp)
        if self.nnz[k]:
            self._chunked(k, buf_ptr, buf_bytes, "rclv", lambda d, m: _lib.call(
                "fh_contacts_scatter", d[0], d[1], d[2], d[3], m, bs_bin, tiles, 0, nbb, C,
                P(self.offsets), P(self.cursor), entries_ptr, sp), stream)

    def rebuild(self):
        """Nothing to do: every walk builds its dataset's segments first."""

    def finish(self):
        pass


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
