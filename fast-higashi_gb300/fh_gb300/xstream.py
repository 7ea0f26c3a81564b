"""X held partly in host memory: the fit when X is larger than its HBM budget.

The fit reads X (every cell's walk output over every band row) twice per ALS iteration, so X
normally stays resident in HBM.  At 50,000 cells, R = 128, band 40 and 500 kb, X is 179 GB in
two bf16 planes (or in fp32), more than a 180 GB budget leaves once the factors, the staging
and the contact segments have their share.  The reference's answer to memory limits is to tile
its work by free GPU memory (bin batches x cell batches, FastHigashi_Wrapper.py:497-517) and
to copy each tile to the device when it is used (sparse_for_schic.py:588-613).  Here the
split is by chromosome and planned once:

* the first chromosomes (in tile order) stay resident: band rows [0, split) in one buffer;
* the rest are grouped into at most four windows of whole chromosomes, each stored in
  page-locked host memory as [planes][cells][ld] (ld = its band rows rounded up to 128, the
  padding zero), exactly the layout a pass over X reads;
* two staging slots in HBM hold two windows at a time.

A pass over X runs the windows already in a slot first, then the resident rows, then the
remaining windows, each copied into the slot that the pass freed first: the copies of the
remaining windows run on a copy stream while the resident rows are being read, and the next
pass starts with the two windows this one ended with.  Both passes of an iteration therefore
move only (windows - 2) windows over the host link, behind the resident pass.  Every copy is
one cudaMemcpyAsync between contiguous buffers, ordered against the kernels by events, so the
30 iterations still capture into one CUDA graph (the copies become memcpy nodes).  X G^T sums
into its output range by range (fh_xg_* with accumulate); X^T E writes each range's rows of W.

The walk writes the streamed chromosomes' X into a slot (with their tile table's band rows
re-based to the window) and copies each window out to its host buffer, then walks the resident
chromosomes.  The contact segments of one dataset at a time live in the staging area too, with
the chunks of its COO on their way in, so the budget holds X's resident part, the staging and
the factors, nothing else.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib

SLOT_ALIGN = 2 << 20          # staging slots start on 2 MiB boundaries


def _up(a, b):
    return -(-int(a) // b) * b


@dataclass
class Window:
    chroms: tuple             # chromosome groups (tile order) held in this window
    x0: int                   # band rows [x0, x1)
    x1: int
    ld: int                   # row stride in its slot and host buffer: x1 - x0 rounded up to 128
    nbytes: int               # planes x cells x ld x element bytes


@dataclass
class XPlan:
    rows: int                 # band rows of X
    split: int                # first streamed band row (rows when nothing streams)
    ld_res: int               # row stride of the resident part (split rounded up to 128)
    res_bytes: int
    windows: list = field(default_factory=list)
    slot_bytes: int = 0       # each of the two staging slots (SLOT_ALIGN multiple)
    staging_bytes: int = 0    # the slots, or the largest contact-segment buffer if larger

    @property
    def streamed_bytes(self):
        return sum(w.nbytes for w in self.windows)

    @property
    def first_streamed_chrom(self):
        return self.windows[0].chroms[0] if self.windows else None


def plan_x(chrom_rows, elem_bytes, n_cells, entries_bytes, budget, max_windows=4,
           chunk_bytes=256 << 20):
    """The split of X between HBM and host memory that streams the fewest bytes.

    chrom_rows: band rows [x0, x1) of each chromosome group in tile order (contiguous, from 0);
    elem_bytes: bytes of one X element over its planes (4: fp32 or two bf16 planes; 2: one);
    entries_bytes: per chromosome group, the largest contact-segment buffer of its datasets
    (8 bytes per contact); budget: bytes for X's resident part and the staging area together.
    Windows are whole chromosome groups; the staging holds two slots of the largest window,
    the largest resident dataset's segments, or a slot plus the largest streamed dataset's
    segments (a streamed chromosome is walked into one slot with its segments beside it), in
    the last two cases with at least chunk_bytes more for the COO chunks of the contact build.
    Raises FHError when no split fits."""
    n = len(chrom_rows)
    if n == 0:
        raise _lib.FHError("plan_x", 1, "no chromosomes")
    rows = int(chrom_rows[-1][1])

    def nbytes(r):
        return _up(r, 128) * n_cells * elem_bytes

    for j in range(n, -1, -1):                    # chromosomes j.. stream
        split = int(chrom_rows[j][0]) if j < n else rows
        res = nbytes(split) if split > 0 else 0
        streamed = list(range(j, n))
        windows = []
        if streamed:
            caps = sorted({nbytes(chrom_rows[b][1] - chrom_rows[a][0])
                           for a in streamed for b in streamed if b >= a})
            for cap in caps:
                windows = []
                cur = None
                for c in streamed:
                    if cur is not None and nbytes(chrom_rows[c][1] - chrom_rows[cur[0]][0]) <= cap:
                        cur.append(c)
                        continue
                    if cur is not None:
                        windows.append(cur)
                    cur = [c]
                windows.append(cur)
                if len(windows) <= max_windows:
                    break
            wins = []
            for g in windows:
                x0, x1 = int(chrom_rows[g[0]][0]), int(chrom_rows[g[-1]][1])
                wins.append(Window(tuple(g), x0, x1, _up(x1 - x0, 128), nbytes(x1 - x0)))
            windows = wins
        slot = _up(max((w.nbytes for w in windows), default=0), SLOT_ALIGN)
        ent_res = max((entries_bytes[c] for c in range(j)), default=0)
        ent_str = max((entries_bytes[c] for c in range(j, n)), default=0)
        need_res = _up(ent_res, SLOT_ALIGN) + chunk_bytes
        need_str = (slot + _up(ent_str, SLOT_ALIGN) + chunk_bytes) if windows else 0
        staging = _up(max(2 * slot, need_res, need_str), SLOT_ALIGN)
        if res + staging <= budget:
            return XPlan(rows, split, _up(split, 128) if split > 0 else 0, res, windows, slot,
                         staging)
    raise _lib.FHError("plan_x", 2, "X (%d band rows x %d cells) does not fit a budget of "
                       "%.1f GB even with every chromosome streamed" % (rows, n_cells, budget / 1e9))


HostBuffer = _lib.HostBuffer


class XStream:
    """The runtime of an XPlan on one device: the resident part, the staging area, the host
    windows, the slots' contents and the copy stream."""

    def __init__(self, plan, planes, n_cells, dtype, device, tiles, tile_ranges):
        """tiles: the engine's tile table (numpy, tile order); tile_ranges[c] = (t0, t1) of
        chromosome group c.  dtype: torch.bfloat16 (planes 1 or 2) or torch.float32."""
        import torch
        self.torch = torch
        self.plan = plan
        self.planes = planes
        self.C = n_cells
        self.dtype = dtype
        self.device = device
        self.elem = torch.tensor([], dtype=dtype).element_size()
        shape = (planes, n_cells, plan.ld_res) if dtype == torch.bfloat16 else (n_cells, plan.ld_res)
        self.res = torch.zeros(shape, dtype=dtype, device=device)
        self.staging = torch.zeros(plan.staging_bytes, dtype=torch.uint8, device=device)
        self.host = [HostBuffer(w.nbytes) for w in plan.windows]
        self.copy = torch.cuda.Stream(device=device)
        # each window's tiles with band rows re-based to the window (the walk's table)
        self.tile_ranges = tile_ranges
        self.win_tiles = []
        self.win_t0 = []
        for w in plan.windows:
            self.win_tiles.append(None)
            self.win_t0.append(tile_ranges[w.chroms[0]][0])
        self.set_tiles(tiles)
        self.slot_win = [None, None]
        self.link_bytes = 0        # host -> device bytes copied so far (windows)

    def set_tiles(self, tiles):
        """(Re)loads each window's tile table from the engine's (epoch counts may change)."""
        torch = self.torch
        for i, w in enumerate(self.plan.windows):
            t0 = self.win_t0[i]
            t1 = self.tile_ranges[w.chroms[-1]][1]
            t = tiles[t0:t1].copy()
            t["xoff"] -= w.x0
            self.win_tiles[i] = torch.from_numpy(t.view(np.uint8).copy()).to(self.device)

    # ------------------------------------------------------------------ layout
    def slot_ptr(self, s):
        return self.staging.data_ptr() + s * self.plan.slot_bytes

    def view(self, s, wi):
        """Slot s holding window wi as a tensor [planes][cells][ld] (or [cells][ld])."""
        w = self.plan.windows[wi]
        n = w.nbytes // self.elem
        off = s * self.plan.slot_bytes // self.elem
        flat = self.staging.view(self.dtype)[off:off + n]
        if self.dtype == self.torch.bfloat16:
            return flat.view(self.planes, self.C, w.ld)
        return flat.view(self.C, w.ld)

    def build_space(self, streamed, entries_bytes):
        """(segments, COO chunk buffer, its bytes) for one dataset's contact build in the
        staging area: from its start for a resident chromosome, after slot 0 for a streamed
        one (whose walk writes slot 0)."""
        start = self.plan.slot_bytes if streamed else 0
        b0 = _up(start + entries_bytes, SLOT_ALIGN)
        return (self.staging.data_ptr() + start, self.staging.data_ptr() + b0,
                self.plan.staging_bytes - b0)

    def window_of_chrom(self, c):
        for i, w in enumerate(self.plan.windows):
            if c in w.chroms:
                return i
        return None

    # ------------------------------------------------------------------ copies
    def reset(self):
        """Forget the slots' contents (after the walk, and before a captured sequence, which
        must not depend on what an earlier one left)."""
        self.slot_win = [None, None]

    def _main(self, stream):
        return stream if stream is not None else self.torch.cuda.current_stream(self.device)

    def _load(self, s, wi, main):
        """Copies window wi into slot s after everything issued on main so far (the last pass
        that used the slot); returns the event that the copy's users wait on."""
        torch = self.torch
        ev = torch.cuda.Event()
        ev.record(main)
        self.copy.wait_event(ev)
        w = self.plan.windows[wi]
        _lib.call("fh_memcpy_async", self.slot_ptr(s), self.host[wi].ptr, w.nbytes,
                  self.copy.cuda_stream)
        done = torch.cuda.Event()
        done.record(self.copy)
        self.slot_win[s] = wi
        self.link_bytes += w.nbytes
        return done

    def hold(self, wi, stream=None):
        """Window wi in a slot (copied in if it is not there yet), ready on the main stream;
        returns its view."""
        main = self._main(stream)
        if wi in self.slot_win:
            return self.view(self.slot_win.index(wi), wi)
        s = 0 if self.slot_win[0] is None else (1 if self.slot_win[1] is None else 0)
        main.wait_event(self._load(s, wi, main))
        return self.view(s, wi)

    def store_window(self, wi, s, stream=None):
        """Copies slot s (window wi, just walked) out to its host buffer; returns the event."""
        torch = self.torch
        main = self._main(stream)
        ev = torch.cuda.Event()
        ev.record(main)
        self.copy.wait_event(ev)
        _lib.call("fh_memcpy_async", self.host[wi].ptr, self.slot_ptr(s),
                  self.plan.windows[wi].nbytes, self.copy.cuda_stream)
        done = torch.cuda.Event()
        done.record(self.copy)
        return done

    def run_pass(self, res_fn, win_fn, stream=None):
        """One pass over X: res_fn(X_res, rows) for the resident rows (if any), win_fn(view,
        window) for each window, in the order that keeps the copies behind the resident rows."""
        main = self._main(stream)
        W = self.plan.windows
        first = [wi for wi in self.slot_win if wi is not None]
        pending = [wi for wi in range(len(W)) if wi not in first]
        rest = list(pending)
        queued = {}
        for s in range(2):                          # empty slots: start their copies now
            if self.slot_win[s] is None and pending:
                wi = pending.pop(0)
                queued[wi] = (s, self._load(s, wi, main))
        for item in first + ["res"] + rest:
            if item == "res":
                if self.plan.split > 0:
                    res_fn(self.res, self.plan.split)
                continue
            wi = item
            if wi in queued:
                s, ev = queued.pop(wi)
                main.wait_event(ev)
            else:
                s = self.slot_win.index(wi)
            win_fn(self.view(s, wi), W[wi])
            if pending:                             # the slot is free once this pass ends
                nxt = pending.pop(0)
                queued[nxt] = (s, self._load(s, nxt, main))
