"""Device-resident fit engine: contact build, RWR once, then the ALS sweep as kernel launches.

The forms share everything but X and the two passes over it:
  precision="fp32"    the plain drop-in: X in fp32, CUDA-core passes (fh_xe_f32 / fh_xg_f32)
  precision="bf16x2"  the tensor-core form: X as two bf16 planes (hi, lo: 16 significant
                      bits), tcgen05 passes (fh_xe_bf16 / fh_xg_bf16) with the small operands
                      split hi|lo as well, so the products are fp32-class; every other step fp32
  precision="bf16"    the same with one bf16 plane (half the X traffic, X rounded to 2^-9)
Layout in HBM (all on one GPU):
  entries   packed contacts, one segment per (bin batch, cell)           8 B / contact
  X / X16   RWR output of every cell: X[cell][band row]              4 B / 2 B per element
            band row = tile.xoff + i * width + j; the row stride is padded to 128
  W, Gt     [band row][rp]: X^T E and the projection rows U M^T
  U         projections, tile-major (rows, width, r) as the reference's projection_list
  Y         [bin row][ld][rp] projected tensors
  A         [bin row][ld];  B [chrom][ld][ld];  D [chrom][rp][ld];  E [cell][rp]
  cov       do_col coverage rows [cell][bin across chromosomes] (good cells, then bad)
Per ALS iteration (parafac2_intergrative.py:635-737): procrustes (per bin row polar) ->
X G^T (SVD_term) -> meta polar (E) -> X^T E (W) -> Y -> CP-ALS sweeps.  Loss scalars go
into a device history and are turned into the reference's rec_error values on the host.
Ranks: R and every chromosome's r up to 128 (rp in {16, 32, 64, 128}; the bf16 forms use
rp >= 32).  The walk's options: do_conv (3 x 3 mean first), do_col (column-normalised walk
over the coverage rows); both run on fp32 CUDA cores and write X in the engine's precision.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .sparse_for_schic import ContactStore, tile_table


def _pad_rank(R):
    for p in (16, 32, 64, 128):
        if R <= p:
            return p
    raise _lib.FHError("engine", 2, "rank %d > 128" % R)


class FitEngine:
    # bytes of a budget kept back for transient buffers (init's sketches, the auto-stop deltas)
    BUDGET_RESERVE = 2 << 30
    # least staging room for the two COO chunk buffers of a budgeted contact build
    BUDGET_CHUNK = 256 << 20

    def __init__(self, schic, rank, chrom2size, n_i, device, do_rwr=True, stream=None,
                 precision="fp32", do_conv=False, do_col=False, bin_cov=None, hbm_budget=None):
        """bin_cov: (bin_cov_list, bad_bin_cov_list) of the model, required with do_col when
        n_i is given (the walk runs at construction); init_params computes it otherwise.
        hbm_budget: bytes of device memory this engine may hold, or None (X and every
        dataset's contact segments resident).  With a budget, the contact segments are built
        one dataset at a time from the host COO (copied in chunks through the staging area),
        and X's last chromosomes stream from host memory when X does not fit (xstream.py)."""
        import torch
        self.torch = torch
        if precision not in ("fp32", "bf16", "bf16x2"):
            raise _lib.FHError("FitEngine", 1, "precision must be 'fp32', 'bf16' or 'bf16x2'")
        self.precision = precision
        self.bf16 = precision != "fp32"
        self.planes = 2 if precision == "bf16x2" else 1
        self.timing = None   # {kernel family: [(start event, end event)]} when enabled
        self._rwr_form = None  # form of the tensor-core walk, tuned at its first run
        # K chunks of 64 per tensor-memory accumulator run in the bf16 X passes (0: the
        # library's default); shorter runs, more compensated folds
        self.fold = 0
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise _lib.FHError("FitEngine", 2, "the fit runs on a CUDA device only")
        _lib.load()
        self.schic = schic
        self.R = int(rank)
        self.rp = _pad_rank(self.R)
        if self.bf16:
            self.rp = max(self.rp, 32)   # the tensor-core passes take N = 2 rp >= 64
        self.ld = self.rp
        self.C = schic[0].num_cell
        self.Ct = schic[0].total_cell_num
        for d in schic:
            if d.num_cell != self.C or d.total_cell_num != self.Ct:
                raise _lib.FHError("FitEngine", 1, "datasets disagree on the cell count")
        self.names = []
        for d in schic:
            if d.chrom not in self.names:
                self.names.append(d.chrom)
        self.chrom_index = [self.names.index(d.chrom) for d in schic]
        # several resolutions: the datasets of a chromosome share its B and D, its CP-ALS runs
        # on their bin rows together, and the per-dataset losses need per-dataset core norms
        self.multi = len(self.names) != len(schic)
        self.ranks = [int(chrom2size[d.chrom]) for d in schic]
        if max(self.ranks) > 128 or self.R > 128:
            raise _lib.FHError("FitEngine", 2, "ranks above 128 are not supported")
        self.do_rwr = do_rwr
        self.do_conv = bool(do_conv)
        self.do_col = bool(do_col) and bool(do_rwr)   # do_col acts inside the walk only
        self._xc = None     # fp32 3 x 3-mean tiles for the bf16 forms (do_conv)
        self.cov = None     # do_col coverage rows [Ct][nb] (bin_cov, then bad_bin_cov rows)
        self.cov_src = None  # the caller's (bin_cov_list, bad_bin_cov_list) the rows came from
        self.n_rwr = [int(v) if do_rwr else 0 for v in (n_i if n_i is not None else [0] * len(schic))]
        order = sorted(range(len(schic)), key=lambda k: self.chrom_index[k])
        self.tiles, self.tile_base = tile_table(schic, self.chrom_index, self.ranks, self.n_rwr, order)
        t = self.tiles
        if (t["width"] < t["rank"]).any():
            # the per-bin polar factors are taken through a QR of the n x r matrix (n >= r)
            raise _lib.FHError("FitEngine", 2,
                               "a bin batch has fewer compact columns than its chromosome's rank")
        self.n_tiles = len(t)
        self.rows = int((t["rows"] * t["width"]).sum())
        self.ldx = int(math.ceil(self.rows / 128) * 128)
        self.ldw = self.ldx                  # rows of W and Gt (all band rows)
        self.nb = int(t["rows"].sum())
        self.max_rows = int(t["rows"].max())
        self.max_width = int(t["width"].max())
        self.max_rank = int(t["rank"].max())
        self.u_size = int((t["rows"] * t["width"] * t["rank"]).sum())
        # bin rows of each dataset and chromosome
        self.ds_rows = []
        for k, d in enumerate(schic):
            t0 = self.tile_base[k]
            b0 = int(t["brow0"][t0])
            self.ds_rows.append(slice(b0, b0 + d.num_bin))
        row_tile = np.repeat(np.arange(self.n_tiles, dtype=np.int32), t["rows"])
        self.stream = stream
        dev = self.device
        f32, f64, i32 = torch.float32, torch.float64, torch.int32
        self.row_tile = torch.from_numpy(row_tile).to(dev)
        self.status = torch.zeros(1, dtype=i32, device=dev)
        self.xs = None
        self.order = order
        if hbm_budget is not None:
            self._budgeted(hbm_budget, n_i)
        else:
            self._resident(n_i, bin_cov)
        self._buffers()

    def _resident(self, n_i, bin_cov):
        """X and every dataset's contact segments in HBM; the walk at construction when n_i
        is given (each dataset's walk right behind its contact build)."""
        torch, dev, order = self.torch, self.device, self.order
        f32, f64 = torch.float32, torch.float64
        # ---- contacts and RWR (once)
        self.store = ContactStore(self.schic, dev, self.tiles, self.tile_base, self.stream,
                                  order=order, defer=True)
        self.tiles_dev = self.store.tiles_dev
        # every walk writes all band rows [0, rows) of X; only the padding columns up to the
        # 128-row stride need zeros once (the passes read them), not all of X
        if self.bf16:
            self.X = None
            self.X16 = torch.empty((self.planes, self.Ct, self.ldx), dtype=torch.bfloat16,
                                   device=dev)
            self.X16[:, :, self.rows:].zero_()
        else:
            self.X = torch.empty((self.Ct, self.ldx), dtype=f32, device=dev)
            self.X[:, self.rows:].zero_()
            self.X16 = None
        self.sumsq = torch.zeros(self.n_tiles * self.Ct, dtype=f64, device=dev)
        if n_i is not None and not (self.do_col or self.do_conv):
            # each dataset's walk starts as soon as its contacts are built, while the next
            # dataset's host-to-device copy is still in flight
            for k in order:
                self.store.build(k)
                self._rwr_dataset(k)
            self.store.finish()
        else:
            self.store.build_all()
            self.store.finish()
            if self.do_col and bin_cov is not None:
                self.set_coverage(*bin_cov)
            if n_i is not None:
                self.run_rwr()

    def _budgeted(self, budget, n_i):
        """The engine within hbm_budget bytes: the factor buffers' share first, then the plan
        of X (xstream.plan_x) over what remains, less a reserve for the transient buffers of
        init and the walk's auto-stop deltas."""
        from .sparse_for_schic import StreamedContacts
        from .xstream import XStream, plan_x
        torch, dev = self.torch, self.device
        if self.do_conv or self.do_col:
            raise _lib.FHError("FitEngine", 2, "do_conv and do_col need X resident "
                                               "(no hbm_budget)")
        self.store = StreamedContacts(self.schic, dev, self.tiles, self.tile_base, self.status,
                                      order=self.order)
        self.tiles_dev = self.store.tiles_dev
        groups = []                          # chromosome groups in tile order: (datasets, t0, t1)
        for ci in range(len(self.names)):
            ks = [k for k in self.order if self.chrom_index[k] == ci]
            t0 = min(self.tile_base[k] for k in ks)
            t1 = max(self.tile_base[k] + self.schic[k].num_bin_batch for k in ks)
            groups.append((ks, t0, t1))
        groups.sort(key=lambda g: g[1])
        t = self.tiles
        chrom_rows = [(int(t["xoff"][t0]), int(t["xoff"][t1 - 1] + t["rows"][t1 - 1] * t["width"][t1 - 1]))
                      for _, t0, t1 in groups]
        entries = [max(self.store.entries_bytes(k) for k in ks) for ks, _, _ in groups]
        elem = 2 * self.planes if self.bf16 else 4
        x_budget = int(budget) - self._buffer_bytes(True) - self.store_bytes() - \
            self.BUDGET_RESERVE
        plan = plan_x(chrom_rows, elem, self.Ct, entries, x_budget, chunk_bytes=self.BUDGET_CHUNK)
        self.groups = groups
        self.xs = XStream(plan, self.planes, self.Ct,
                          torch.bfloat16 if self.bf16 else torch.float32, dev, self.tiles,
                          [(t0, t1) for _, t0, t1 in groups])
        self.ldx = plan.ld_res
        if self.bf16:
            self.X, self.X16 = None, self.xs.res
        else:
            self.X, self.X16 = self.xs.res, None
        self.sumsq = torch.zeros(self.n_tiles * self.Ct, dtype=torch.float64, device=dev)
        if n_i is not None:
            self.run_rwr()

    def store_bytes(self):
        s = self.store
        return s.counts.numel() * 8 + s.offsets.numel() * 8 + s.scan_ws.numel()

    def _partial_splits(self, budgeted=None):
        if budgeted if budgeted is not None else self.xs is not None:
            # the streamed passes take the heuristic split count of each row range
            return max(self.xg_splits(self.C, self.rows), self.xg_splits(self.Ct, self.rows))
        # room for the autotuner's largest split candidate (four times the heuristic)
        return 4 * max(self.xg_splits(self.C, self.rows), self.xg_splits(self.Ct, self.rows))

    def _buffer_bytes(self, budgeted=None):
        """Bytes of the factor state and work buffers that _buffers allocates."""
        nchrom, ld, rp, C, Ct = len(self.names), self.ld, self.rp, self.C, self.Ct
        b = 4 * (self.nb * ld + nchrom * ld * ld + nchrom * rp * ld + C * rp)
        b += 4 * 2 * self.ldw * rp + 4 * max(self.u_size, 1) + 4 * self.nb * ld * rp
        b += 4 * Ct * rp + 4 * self._partial_splits(budgeted) * Ct * rp + 8 * (self.nb + 1 + nchrom)
        if self.bf16:
            b += 2 * Ct * 2 * rp + 2 * self.rows * 2 * rp
        b += _lib.value("fh_meta_polar_workspace", Ct, self.R)
        b += 8 * self.n_tiles * Ct                  # sumsq
        return b

    def _buffers(self):
        """Factor state and work buffers."""
        torch, dev = self.torch, self.device
        f32, f64 = torch.float32, torch.float64
        # ---- factor state and work buffers
        nchrom = len(self.names)
        self.A = torch.zeros((self.nb, self.ld), dtype=f32, device=dev)
        self.B = torch.zeros((nchrom, self.ld, self.ld), dtype=f32, device=dev)
        self.D = torch.zeros((nchrom, self.rp, self.ld), dtype=f32, device=dev)
        self.E = torch.zeros((self.C, self.rp), dtype=f32, device=dev)
        self.W = torch.zeros((self.ldw, self.rp), dtype=f32, device=dev)
        self.Gt = torch.zeros((self.ldw, self.rp), dtype=f32, device=dev)
        self.U = torch.zeros(max(self.u_size, 1), dtype=f32, device=dev)
        self.Y = torch.zeros((self.nb, self.ld, self.rp), dtype=f32, device=dev)
        self.S = torch.zeros((self.Ct, self.rp), dtype=f32, device=dev)
        self.splits = self._partial_splits()
        self._tuned = {}
        if self.bf16:
            self.E2 = torch.zeros((self.Ct, 2 * self.rp), dtype=torch.bfloat16, device=dev)
            self.G2 = torch.zeros((self.rows, 2 * self.rp), dtype=torch.bfloat16, device=dev)
        self.partial = torch.empty((self.splits, self.Ct, self.rp), dtype=f32, device=dev)
        self.ssum = torch.zeros(self.nb, dtype=f64, device=dev)
        self.meta_ssum = torch.zeros(1, dtype=f64, device=dev)
        self.core = torch.zeros(nchrom, dtype=f64, device=dev)
        mw = _lib.value("fh_meta_polar_workspace", self.Ct, self.R)
        self.meta_ws = torch.empty(mw, dtype=torch.uint8, device=dev)
        # CP-ALS chunk tables (<= 8 rows of one chromosome; the autotuner may pick 4 or 16)
        self._cp_tables = {}
        self.cp_meta, self.nchunks = self.cp_table(8)
        n_most = self.cp_table(4)[1]
        cw = _lib.value("fh_cp_workspace", nchrom, n_most, self.ld, self.rp)
        self.cp_ws = torch.empty(cw, dtype=torch.uint8, device=dev)
        self._cp_tuned = False
        self.history = []

    # ------------------------------------------------------------------ helpers
    def sp(self):
        return _lib.stream_ptr(self.stream)

    def _timed(self, name, fn):
        """Runs fn; with timing enabled, brackets it with CUDA events on the launch stream."""
        if self.timing is None:
            return fn()
        torch = self.torch
        stream = self.stream if self.stream is not None else torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        self.timing.setdefault(name, []).append((a, b))
        return out

    def timing_summary(self):
        """Mean milliseconds and launch count per kernel family (after a synchronize)."""
        out = {}
        for k, evs in (self.timing or {}).items():
            ms = [a.elapsed_time(b) for a, b in evs]
            out[k] = dict(mean_ms=float(np.mean(ms)), total_ms=float(np.sum(ms)), calls=len(ms))
        return out

    def check_status(self, what):
        st = int(self.status.item())
        if st:
            self.status.zero_()
            raise _lib.FHError(what, st)

    def set_epochs(self, per_tile):
        """Sets the RWR epoch count of every tile (force_rwr_epochs) and re-uploads the table."""
        self.tiles["n_rwr"] = np.asarray(per_tile, dtype=np.int32)
        self.tiles_dev.copy_(self.torch.from_numpy(self.tiles.view(np.uint8).copy()))
        if self.xs is not None:
            self.xs.set_tiles(self.tiles)

    def set_n_i(self, n_i):
        self.n_rwr = [int(v) if self.do_rwr else 0 for v in n_i]
        per_tile = np.zeros(self.n_tiles, dtype=np.int32)
        for k, d in enumerate(self.schic):
            per_tile[self.tile_base[k]:self.tile_base[k] + d.num_bin_batch] = self.n_rwr[k]
        self.set_epochs(per_tile)

    def auto_deltas(self, cap, all_cells=False):
        """||Q_e - Q_{e+1}||_F for e < cap for every (tile, good cell), or every cell with
        all_cells (partial_rwr.py:99-123)."""
        P = _lib.ptr
        out = self.torch.zeros((self.n_tiles, self.Ct, cap), dtype=self.torch.float32,
                               device=self.device)
        if self.xs is not None:
            # one dataset's segments at a time, at the start of the staging area
            main = self.stream if self.stream is not None else \
                self.torch.cuda.current_stream(self.device)
            for k in self.order:
                tb, nbb = self.tile_base[k], self.schic[k].num_bin_batch
                ent, buf, nbuf = self.xs.build_space(False, self.store.entries_bytes(k))
                self.store.build(k, ent, main, buf, nbuf)
                _lib.call("fh_rwr_tiles_deltas", P(self.tiles_dev) + tb * _lib.TILE_DTYPE.itemsize,
                          nbb, self.Ct, self.max_rows, self.max_width, ent,
                          P(self.store.offsets), cap, P(out) + tb * self.Ct * cap * 4,
                          P(self.status), self.sp())
        elif self.do_conv:
            src = self.conv_source()
            _lib.call("fh_rwr_tiles_dense_deltas", P(self.tiles_dev), self.n_tiles, self.Ct,
                      self.max_rows, self.max_width, P(src), self.ldx, cap, P(out),
                      P(self.status), self.sp())
        else:
            _lib.call("fh_rwr_tiles_deltas", P(self.tiles_dev), self.n_tiles, self.Ct,
                      self.max_rows, self.max_width, P(self.store.entries),
                      P(self.store.offsets), cap, P(out), P(self.status), self.sp())
        return out if all_cells else out[:, :self.C]

    def conv_source(self):
        """The 3 x 3 mean of every floored tile (do_conv, partial_rwr.py:79-83) in the X layout:
        into X itself in the fp32 form (the walk then runs in place), into a scratch fp32
        array in the bf16 forms."""
        if self.bf16:
            if self._xc is None:
                self._xc = self.torch.empty((self.Ct, self.ldx), dtype=self.torch.float32,
                                            device=self.device)
            buf = self._xc
        else:
            buf = self.X
        P = _lib.ptr
        _lib.call("fh_conv_tiles_f32", P(self.tiles_dev), self.n_tiles, self.Ct, self.max_rows,
                  self.max_width, P(self.store.entries), P(self.store.offsets), P(buf), self.ldx,
                  P(self.status), self.sp())
        return buf

    # ------------------------------------------------------------------ do_col
    def set_coverage(self, good, bad):
        """Coverage rows from the model's bin_cov_list (per dataset [num_cell][num_bin]) and
        bad_bin_cov_list (per dataset [bad cells][num_bin], or 0 without bad cells)."""
        torch = self.torch
        if self.cov is None:
            self.cov = torch.ones((self.Ct, self.nb), dtype=torch.float32, device=self.device)
        for k in range(len(self.schic)):
            cols = self.ds_rows[k]
            self.cov[:self.C, cols] = torch.as_tensor(good[k]).to(self.device, torch.float32)
            if self.Ct > self.C and not np.isscalar(bad[k]):
                self.cov[self.C:, cols] = torch.as_tensor(bad[k]).to(self.device, torch.float32)

    def coverage_views(self):
        """(bin_cov_list, bad_bin_cov_list) as views of the coverage rows."""
        good = [self.cov[:self.C, self.ds_rows[k]] for k in range(len(self.schic))]
        bad = [self.cov[self.C:, self.ds_rows[k]] if self.Ct > self.C else 0
               for k in range(len(self.schic))]
        return good, bad

    def _col_walk(self, cov, cell_epochs=None, to_x=True, colsum=None):
        P = _lib.ptr
        dense = self.conv_source() if self.do_conv else None
        _lib.call("fh_rwr_col_tiles", P(self.tiles_dev), self.n_tiles, self.Ct, self.max_rows,
                  self.max_width, P(self.store.entries), P(self.store.offsets),
                  P(dense) if dense is not None else None,
                  P(cov) if cov is not None else None, self.nb,
                  P(cell_epochs) if cell_epochs is not None else None,
                  P(self.X) if to_x and not self.bf16 else None,
                  P(self.X16) if to_x and self.bf16 else None, self.ldx,
                  self.Ct * self.ldx if self.planes == 2 else 0,
                  P(self.sumsq) if to_x else None, P(colsum) if colsum is not None else None,
                  P(self.status), self.sp())

    def compute_coverage(self, cell_epochs):
        """init_params' coverage rows (parafac2_intergrative.py:96-142, 186-200) for all cells:
        1e-4 plus the column sums of the auto-stopped plain walk (cell_epochs: int32 [tile]
        [Ct] per cell batch), added in bin-batch order.  Not yet marked inf."""
        torch, P = self.torch, _lib.ptr
        ep = torch.as_tensor(np.ascontiguousarray(cell_epochs, dtype=np.int32)).to(self.device)
        colsum = torch.empty((self.n_tiles, self.Ct, self.max_width), dtype=torch.float32,
                             device=self.device)
        self._col_walk(None, ep, to_x=False, colsum=colsum)
        if self.cov is None:
            self.cov = torch.empty((self.Ct, self.nb), dtype=torch.float32, device=self.device)
        _lib.call("fh_col_coverage", P(self.tiles_dev), self.n_tiles, self.Ct, P(colsum),
                  self.max_width, P(self.cov), self.nb, self.nb, P(self.status), self.sp())
        del colsum
        self.cov_src = None

    def col_features(self, cell_epochs):
        """The do_col walk with per-cell-batch epochs (the init feature pass, :203-240)."""
        ep = self.torch.as_tensor(np.ascontiguousarray(cell_epochs, dtype=np.int32)).to(self.device)
        self._timed("rwr", lambda: self._col_walk(self.cov, ep))

    def finalize_coverage(self):
        """bin_cov[bin_cov <= 1e-4] = inf (parafac2_intergrative.py:266-270)."""
        _lib.call("fh_col_coverage_finalize", _lib.ptr(self.cov), self.cov.numel(), self.sp())

    def run_rwr(self):
        self._timed("rwr", self._run_rwr)

    def _run_rwr(self):
        P = _lib.ptr
        if self.xs is not None:
            self._walk_streamed()
            return
        if self.do_col:
            if self.cov is None:
                raise _lib.FHError("FitEngine", 1, "do_col needs the coverage rows (bin_cov_list)")
            self._col_walk(self.cov)
            return
        if self.do_conv:
            # the walk from the smoothed tiles (fp32 CUDA cores in every form)
            src = self.conv_source()
            if self.bf16:
                _lib.call("fh_rwr_tiles_dense_bf16", P(self.tiles_dev), self.n_tiles, self.Ct,
                          self.max_rows, self.max_width, P(src), P(self.X16), self.ldx,
                          self.Ct * self.ldx if self.planes == 2 else 0, P(self.sumsq),
                          P(self.status), self.sp())
            else:
                _lib.call("fh_rwr_tiles_dense_f32", P(self.tiles_dev), self.n_tiles, self.Ct,
                          self.max_rows, self.max_width, P(src), P(self.X), self.ldx,
                          P(self.sumsq), P(self.status), self.sp())
            return
        if self.bf16 and self.max_rows <= 128 and self.max_width <= 256:
            self._rwr_tc(self.tuned_rwr_form())
        elif self.bf16:
            _lib.call("fh_rwr_tiles_bf16", P(self.tiles_dev), self.n_tiles, self.Ct,
                      self.max_rows, self.max_width, P(self.store.entries),
                      P(self.store.offsets), P(self.X16), self.ldx,
                      self.Ct * self.ldx if self.planes == 2 else 0, P(self.sumsq),
                      P(self.status), self.sp())
        else:
            _lib.call("fh_rwr_tiles_f32", P(self.tiles_dev), self.n_tiles, self.Ct,
                      self.max_rows, self.max_width, P(self.store.entries),
                      P(self.store.offsets), P(self.X), self.ldx, P(self.sumsq),
                      P(self.status), self.sp())

    def _rwr_dataset(self, k):
        """The plain walk of dataset k's tiles alone (its slice of the tile table, offsets and
        sums; X rows are absolute), in the form the full walk would use."""
        P = _lib.ptr
        tb, nbb = self.tile_base[k], self.schic[k].num_bin_batch
        tiles = P(self.tiles_dev) + tb * _lib.TILE_DTYPE.itemsize
        offs = P(self.store.offsets) + tb * self.Ct * 8
        ss = P(self.sumsq) + tb * self.Ct * 8
        if self.bf16 and self.max_rows <= 128 and self.max_width <= 256:
            form = self._rwr_form or self.cached_rwr_form() or 1
            _lib.call("fh_rwr_tiles_tc", tiles, nbb, self.Ct, self.max_rows, self.max_width,
                      P(self.store.entries), offs, P(self.X16), self.ldx,
                      self.Ct * self.ldx if self.planes == 2 else 0, ss, int(form),
                      P(self.status), self.sp())
        elif self.bf16:
            _lib.call("fh_rwr_tiles_bf16", tiles, nbb, self.Ct, self.max_rows, self.max_width,
                      P(self.store.entries), offs, P(self.X16), self.ldx,
                      self.Ct * self.ldx if self.planes == 2 else 0, ss, P(self.status),
                      self.sp())
        else:
            _lib.call("fh_rwr_tiles_f32", tiles, nbb, self.Ct, self.max_rows, self.max_width,
                      P(self.store.entries), offs, P(self.X), self.ldx, ss, P(self.status),
                      self.sp())

    def _walk_dataset(self, k, X, ldx, tiles_ptr, entries_ptr):
        """The plain walk of dataset k (budgeted engine): its segments at entries_ptr with
        the store's dataset-local offsets, its tiles at tiles_ptr (band rows relative to X's
        column 0), X [planes][cells][ldx] or [cells][ldx]."""
        P = _lib.ptr
        tb, nbb = self.tile_base[k], self.schic[k].num_bin_batch
        ss = P(self.sumsq) + tb * self.Ct * 8
        offs = P(self.store.offsets)
        pst = self.Ct * ldx if self.planes == 2 else 0
        if self.bf16 and self.max_rows <= 128 and self.max_width <= 256:
            form = self._rwr_form or self.cached_rwr_form() or 1
            if form == 2 and self.max_width > 192:
                form = 1
            _lib.call("fh_rwr_tiles_tc", tiles_ptr, nbb, self.Ct, self.max_rows, self.max_width,
                      entries_ptr, offs, P(X), ldx, pst, ss, int(form), P(self.status), self.sp())
        elif self.bf16:
            _lib.call("fh_rwr_tiles_bf16", tiles_ptr, nbb, self.Ct, self.max_rows,
                      self.max_width, entries_ptr, offs, P(X), ldx, pst, ss, P(self.status),
                      self.sp())
        else:
            _lib.call("fh_rwr_tiles_f32", tiles_ptr, nbb, self.Ct, self.max_rows, self.max_width,
                      entries_ptr, offs, P(X), ldx, ss, P(self.status), self.sp())

    def _walk_streamed(self):
        """The walk of a budgeted engine.  The streamed windows first: each window's datasets
        are walked into slot 0 (zeroed, so its padding columns are zero) with their segments
        beside it, and the slot is copied out to the window's host buffer on the copy stream;
        then the resident chromosomes, their segments at the start of the staging area (after
        the last copy-out has read slot 0)."""
        torch, P = self.torch, _lib.ptr
        xs = self.xs
        main = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        xs.reset()
        last = None
        for wi, w in enumerate(xs.plan.windows):
            if last is not None:
                main.wait_event(last)
            view = xs.view(0, wi)
            with torch.cuda.stream(main):
                view.zero_()
            for c in w.chroms:
                for k in self.groups[c][0]:
                    tiles = P(xs.win_tiles[wi]) + (self.tile_base[k] - xs.win_t0[wi]) * \
                        _lib.TILE_DTYPE.itemsize
                    ent, buf, nbuf = xs.build_space(True, self.store.entries_bytes(k))
                    self._timed("contacts", lambda: self.store.build(k, ent, main, buf, nbuf))
                    self._walk_dataset(k, view, w.ld, tiles, ent)
            last = xs.store_window(wi, 0, main)
        if last is not None:
            main.wait_event(last)
        n_res = xs.plan.first_streamed_chrom
        n_res = len(self.groups) if n_res is None else n_res
        for c in range(n_res):
            for k in self.groups[c][0]:
                ent, buf, nbuf = xs.build_space(False, self.store.entries_bytes(k))
                self._timed("contacts", lambda: self.store.build(k, ent, main, buf, nbuf))
                self._walk_dataset(k, xs.res, xs.plan.ld_res,
                                   P(self.tiles_dev) + self.tile_base[k] * _lib.TILE_DTYPE.itemsize,
                                   ent)
        xs.reset()

    def _rwr_signature(self):
        return (self.precision, self.Ct, self.n_tiles, self.max_width,
                int(np.asarray(self.tiles["n_rwr"]).max()))

    def cached_rwr_form(self):
        """The tuner's earlier choice of the walk's form for this shape, without tuning."""
        from . import autotune
        dev = self.torch.cuda.get_device_name(self.device)
        return autotune.default_tuner().lookup(dev, "rwr_form", self._rwr_signature())

    def _rwr_tc(self, form):
        P = _lib.ptr
        _lib.call("fh_rwr_tiles_tc", P(self.tiles_dev), self.n_tiles, self.Ct, self.max_rows,
                  self.max_width, P(self.store.entries), P(self.store.offsets), P(self.X16),
                  self.ldx, self.Ct * self.ldx if self.planes == 2 else 0, P(self.sumsq),
                  int(form), P(self.status), self.sp())

    def tuned_rwr_form(self):
        """Form of the tensor-core walk (fh_rwr_tiles_tc): the autotuner's pick between P in
        shared memory (1, the default) and the block-pipelined form with P in tensor memory
        (2, tiles up to 192 columns), timed on this engine's own tiles at the first call."""
        if self._rwr_form is None:
            if self.max_width > 192 or self.torch.cuda.is_current_stream_capturing():
                return 1
            from . import autotune
            dev = self.torch.cuda.get_device_name(self.device)
            self._rwr_form = autotune.default_tuner().choose(dev, "rwr_form",
                                                             self._rwr_signature(), [1, 2],
                                                             self._rwr_tc, reps=1)
        return self._rwr_form

    # ------------------------------------------------------------------ X passes
    def xg_splits(self, n_cells, rows):
        name = "fh_xg_bf16_splits" if self.bf16 else "fh_xg_splits"
        return _lib.value(name, n_cells, rows)

    def x_rows(self, x0, x1):
        """A view of X holding band rows [x0, x1): (tensor, row stride, band row of its column
        0).  X itself when it is resident; with a budget, the resident part or the slot that
        holds the window of those rows (copied in if needed; [x0, x1) within one chromosome
        group's rows)."""
        if self.xs is None:
            return (self.X16 if self.bf16 else self.X), self.ldx, 0
        plan = self.xs.plan
        if x1 <= plan.split:
            return self.xs.res, plan.ld_res, 0
        for wi, w in enumerate(plan.windows):
            if w.x0 <= x0 and x1 <= w.x1:
                return self.xs.hold(wi, self.stream), w.ld, w.x0
        raise _lib.FHError("x_rows", 1, "rows [%d, %d) span a streamed window's edge" % (x0, x1))

    def x_times_e(self, a0, rows, n_cells, E, rp, W, E2=None, view=None):
        """W[row][m] = sum_{c < n_cells} X[c][a0 + row] E[c][m]  (E: [n_cells][rp] fp32,
        W: [rows][rp]); a0 is a multiple of 128.  view: (X tensor, row stride) from x_rows
        (default: X itself)."""
        P = _lib.ptr
        X, ld = view if view is not None else ((self.X16 if self.bf16 else self.X), self.ldx)
        if self.bf16:
            if E2 is None:
                E2 = self.torch.empty((n_cells, 2 * rp), dtype=self.torch.bfloat16,
                                      device=self.device)
            _lib.call("fh_split_bf16", P(E), n_cells, rp, rp, P(E2), self.sp())
            _lib.call("fh_xe_bf16", P(X[0, :, a0:]), ld, self.Ct, self.planes, n_cells, rows,
                      P(E2), rp, self.fold, P(W), P(self.status), self.sp())
        else:
            _lib.call("fh_xe_f32", P(X[:, a0:]), ld, n_cells, rows, P(E), rp, P(W), self.sp())

    def x_times_g(self, a0, rows, n_cells, Gt, rp, splits, partial, out, G2=None, view=None):
        """out[c][m] = sum_row X[c][a0 + row] Gt[row][m] for c < n_cells (Gt: [rows][rp]).
        view: as for x_times_e."""
        P = _lib.ptr
        X, ld = view if view is not None else ((self.X16 if self.bf16 else self.X), self.ldx)
        if self.bf16:
            if G2 is None:
                G2 = self.torch.empty((rows, 2 * rp), dtype=self.torch.bfloat16,
                                      device=self.device)
            _lib.call("fh_split_bf16", P(Gt), rows, rp, rp, P(G2), self.sp())
            _lib.call("fh_xg_bf16", P(X[0, :, a0:]), ld, self.Ct, self.planes, n_cells, rows,
                      P(G2), rp, splits, self.fold, P(partial), P(out), 0, P(self.status),
                      self.sp())
        else:
            _lib.call("fh_xg_f32", P(X[:, a0:]), ld, n_cells, rows, P(Gt), rp, splits,
                      P(partial), P(out), 0, self.sp())

    def _stream_xe(self, n_cells, E, rp, W, E2):
        """W = X^T E over every band row of a budgeted engine: E split once, then one pass per
        row range (resident rows, then each window at its rows of W)."""
        P = _lib.ptr
        sp = self.sp()
        if self.bf16:
            _lib.call("fh_split_bf16", P(E), n_cells, rp, rp, P(E2), sp)

        def seg(X, ld, x0, rows):
            w = P(W) + x0 * rp * 4
            if self.bf16:
                _lib.call("fh_xe_bf16", P(X), ld, self.Ct, self.planes, n_cells, rows, P(E2), rp,
                          self.fold, w, P(self.status), sp)
            else:
                _lib.call("fh_xe_f32", P(X), ld, n_cells, rows, P(E), rp, w, sp)

        self.xs.run_pass(lambda X, rows: seg(X, self.xs.plan.ld_res, 0, rows),
                         lambda X, w: seg(X, w.ld, w.x0, w.x1 - w.x0), self.stream)

    def _stream_xg(self, n_cells, Gt, rp, out, G2):
        """out = X Gt over every band row of a budgeted engine: Gt split once; the first row
        range writes out, the others add into it."""
        P = _lib.ptr
        sp = self.sp()
        if self.bf16:
            _lib.call("fh_split_bf16", P(Gt), self.rows, rp, rp, P(G2), sp)
        first = [True]

        def seg(X, ld, x0, rows):
            acc = 0 if first[0] else 1
            first[0] = False
            splits = min(self.xg_splits(n_cells, rows), self.partial.shape[0])
            if self.bf16:
                _lib.call("fh_xg_bf16", P(X), ld, self.Ct, self.planes, n_cells, rows,
                          P(G2) + x0 * 2 * rp * 2, rp, splits, self.fold, P(self.partial),
                          P(out), acc, P(self.status), sp)
            else:
                _lib.call("fh_xg_f32", P(X), ld, n_cells, rows, P(Gt) + x0 * rp * 4, rp, splits,
                          P(self.partial), P(out), acc, sp)

        self.xs.run_pass(lambda X, rows: seg(X, self.xs.plan.ld_res, 0, rows),
                         lambda X, w: seg(X, w.ld, w.x0, w.x1 - w.x0), self.stream)

    def tensor_norms(self):
        """||X||^2 per dataset over the good-QC cells (parafac2_intergrative.py:369)."""
        s = self.sumsq.view(self.n_tiles, self.Ct)[:, :self.C].sum(1).cpu().numpy()
        out = np.zeros(len(self.schic))
        for k, d in enumerate(self.schic):
            t0 = self.tile_base[k]
            out[k] = s[t0:t0 + d.num_bin_batch].sum()
        return out

    # ------------------------------------------------------------------ state
    def set_state(self, A_list, B_dict, D_dict, E):
        """Loads factors (they may be views of this engine's own buffers)."""
        torch = self.torch
        dev, f32 = self.device, torch.float32
        A_in = [torch.as_tensor(a, dtype=f32).to(dev).clone() for a in A_list]
        B_in = {n: torch.as_tensor(B_dict[n], dtype=f32).to(dev).clone() for n in self.names}
        D_in = {n: torch.as_tensor(D_dict[n], dtype=f32).to(dev).clone() for n in self.names}
        E_in = torch.as_tensor(E, dtype=f32).to(dev).clone()
        self.A.zero_(); self.B.zero_(); self.D.zero_(); self.E.zero_()
        for k, d in enumerate(self.schic):
            self.A[self.ds_rows[k], :self.ranks[k]] = A_in[k]
        for ci, name in enumerate(self.names):
            r = self.ranks[self.chrom_index.index(ci)]
            self.B[ci, :r, :r] = B_in[name]
            self.D[ci, :self.R, :r] = D_in[name]
        self.E[:, :self.R] = E_in[:self.C]

    def A_views(self):
        return [self.A[self.ds_rows[k], :self.ranks[k]] for k in range(len(self.schic))]

    def B_views(self):
        return {n: self.B[ci, :self.ranks[self.chrom_index.index(ci)], :self.ranks[self.chrom_index.index(ci)]]
                for ci, n in enumerate(self.names)}

    def D_views(self):
        return {n: self.D[ci, :self.R, :self.ranks[self.chrom_index.index(ci)]]
                for ci, n in enumerate(self.names)}

    def projection_views(self):
        """U per dataset and bin batch as (b, n, r) tensors (projection_list)."""
        out = []
        for k, d in enumerate(self.schic):
            lst = []
            for bi in range(d.num_bin_batch):
                t = self.tiles[self.tile_base[k] + bi]
                n = int(t["rows"]) * int(t["width"]) * int(t["rank"])
                lst.append(self.U[int(t["uoff"]):int(t["uoff"]) + n].view(int(t["rows"]), int(t["width"]), int(t["rank"])))
            out.append(lst)
        return out

    def projected_views(self):
        """projected_tensor_list: Y per chromosome over all its datasets' bin rows."""
        return {n: self.Y[self.chrom_rows(ci), :self.ranks[self.chrom_index.index(ci)], :self.R]
                for ci, n in enumerate(self.names)}

    # ------------------------------------------------------------------ kernels
    def xe(self):
        if self.xs is not None:
            self._timed("xe", lambda: self._stream_xe(self.C, self.E, self.rp, self.W,
                                                      self.E2[:self.C] if self.bf16 else None))
            return
        self._timed("xe", lambda: self.x_times_e(0, self.rows, self.C, self.E, self.rp, self.W,
                                                 self.E2[:self.C] if self.bf16 else None))

    def procrustes(self):
        P = _lib.ptr
        self._timed("procrustes", lambda: _lib.call(
            "fh_procrustes_f32", P(self.tiles_dev), P(self.row_tile), self.nb, self.max_width,
            self.max_rank, P(self.W), P(self.A), self.ld, P(self.B), P(self.D), self.ld, self.R,
            self.rp, P(self.U), P(self.Gt), P(self.ssum), P(self.status), self.sp()))

    def tuned_splits(self, n_cells):
        """Split count of the X G^T pass over n_cells: the autotuner's pick among the
        heuristic, half, twice and four times it (autotune.py), timed on this engine's own
        buffers at the first call (an eager one: graph capture comes after the first pass)."""
        if n_cells not in self._tuned and self.torch.cuda.is_current_stream_capturing():
            return self.xg_splits(n_cells, self.rows)
        if n_cells not in self._tuned:
            from . import autotune
            h = self.xg_splits(n_cells, self.rows)
            cands = [h] + [v for v in (max(1, h // 2), 2 * h, 4 * h) if v <= self.partial.shape[0]]
            sig = (self.precision, n_cells, self.rows, self.rp)
            dev = self.torch.cuda.get_device_name(self.device)
            self._tuned[n_cells] = autotune.default_tuner().choose(
                dev, "xg_splits", sig, cands,
                lambda v: self.x_times_g(0, self.rows, n_cells, self.Gt, self.rp, v, self.partial,
                                         self.S, self.G2 if self.bf16 else None))
        return self._tuned[n_cells]

    def xg(self, n_cells):
        if self.xs is not None:
            self._timed("xg", lambda: self._stream_xg(n_cells, self.Gt, self.rp, self.S,
                                                      self.G2 if self.bf16 else None))
            return
        splits = self.tuned_splits(n_cells)
        self._timed("xg", lambda: self.x_times_g(0, self.rows, n_cells, self.Gt, self.rp,
                                                 splits, self.partial, self.S,
                                                 self.G2 if self.bf16 else None))

    def meta_polar(self, n_cells, E_out):
        P = _lib.ptr
        self._timed("meta_polar", lambda: _lib.call(
            "fh_meta_polar", P(self.S), n_cells, self.R, self.rp, P(E_out), P(self.meta_ssum),
            P(self.meta_ws), self.meta_ws.numel(), P(self.status), self.sp()))

    def project_y(self):
        P = _lib.ptr
        self._timed("project_y", lambda: _lib.call(
            "fh_project_y_f32", P(self.tiles_dev), P(self.row_tile), self.nb, P(self.U),
            P(self.W), self.rp, P(self.Y), self.ld, self.sp()))

    def chrom_rows(self, ci):
        """Bin rows of chromosome ci: its datasets' rows, adjacent in the row order."""
        ks = [k for k in range(len(self.schic)) if self.chrom_index[k] == ci]
        start = min(self.ds_rows[k].start for k in ks)
        stop = max(self.ds_rows[k].stop for k in ks)
        if stop - start != sum(self.ds_rows[k].stop - self.ds_rows[k].start for k in ks):
            raise _lib.FHError("FitEngine", 2, "a chromosome's datasets are not adjacent")
        return slice(start, stop)

    def dataset_cores(self):
        """core[k] = ||[[A_k, B, D]]||^2 per dataset (parafac2_intergrative.py:697-706) when a
        chromosome has several datasets: fh_core_norm over a table of the datasets' rows, with
        each dataset's B and D gathered from its chromosome's."""
        torch, P = self.torch, _lib.ptr
        if not hasattr(self, "_ds_core"):
            n = len(self.schic)
            c_row0, c_nbin, c_rank, c_chunk0, c_nchunk = [], [], [], [], []
            k_chrom, k_row0, k_nrow = [], [], []
            for k in range(n):
                rs = self.ds_rows[k]
                c_row0.append(rs.start); c_nbin.append(rs.stop - rs.start)
                c_rank.append(self.ranks[k]); c_chunk0.append(len(k_chrom))
                for r0 in range(rs.start, rs.stop, 8):
                    k_chrom.append(k); k_row0.append(r0); k_nrow.append(min(8, rs.stop - r0))
                c_nchunk.append(len(k_chrom) - c_chunk0[-1])
            meta = np.array(c_row0 + c_nbin + c_rank + c_chunk0 + c_nchunk + k_chrom + k_row0 +
                            k_nrow, dtype=np.int32)
            idx = torch.as_tensor(self.chrom_index, dtype=torch.long, device=self.device)
            ws = torch.empty(_lib.value("fh_cp_workspace", n, len(k_chrom), self.ld, self.rp),
                             dtype=torch.uint8, device=self.device)
            self._ds_core = dict(meta=torch.from_numpy(meta).to(self.device), nch=len(k_chrom),
                                 idx=idx, ws=ws,
                                 B=torch.zeros((n, self.ld, self.ld), dtype=torch.float32,
                                               device=self.device),
                                 D=torch.zeros((n, self.rp, self.ld), dtype=torch.float32,
                                               device=self.device))
            self.core_ds = torch.zeros(n, dtype=torch.float64, device=self.device)
        c = self._ds_core
        torch.index_select(self.B, 0, c["idx"], out=c["B"])
        torch.index_select(self.D, 0, c["idx"], out=c["D"])
        _lib.call("fh_core_norm", len(self.schic), c["nch"], P(c["meta"]), P(self.A), P(c["B"]),
                  P(c["D"]), P(self.Y), self.ld, self.rp, self.R, self.ld, P(self.core_ds),
                  P(c["ws"]), c["ws"].numel(), P(self.status), self.sp())

    def cp_table(self, rows):
        """CP-ALS chunk table: chunks of <= rows bin rows inside one chromosome, as the int32
        meta block of fh_cp_als (cached per size).  Returns (device tensor, number of chunks)."""
        if rows not in self._cp_tables:
            c_row0, c_nbin, c_rank, c_chunk0, c_nchunk = [], [], [], [], []
            k_chrom, k_row0, k_nrow = [], [], []
            for ci, name in enumerate(self.names):
                k = self.chrom_index.index(ci)
                rs = self.chrom_rows(ci)
                c_row0.append(rs.start); c_nbin.append(rs.stop - rs.start)
                c_rank.append(self.ranks[k]); c_chunk0.append(len(k_chrom))
                for r0 in range(rs.start, rs.stop, rows):
                    k_chrom.append(ci); k_row0.append(r0); k_nrow.append(min(rows, rs.stop - r0))
                c_nchunk.append(len(k_chrom) - c_chunk0[-1])
            meta = np.array(c_row0 + c_nbin + c_rank + c_chunk0 + c_nchunk + k_chrom + k_row0 +
                            k_nrow, dtype=np.int32)
            self._cp_tables[rows] = (self.torch.from_numpy(meta).to(self.device), len(k_chrom))
        return self._cp_tables[rows]

    def tune_cp(self):
        """Chunk size of the CP-ALS row kernels (bin rows per CTA): the autotuner times one
        sweep for 8 (the default), 4 and 16 rows on the current factors, restoring them after
        each run, and keeps the fastest.  Runs at the first CP-ALS call (an eager one)."""
        self._cp_tuned = True
        if self.torch.cuda.is_current_stream_capturing():
            return
        from . import autotune
        P = _lib.ptr
        state = (self.A, self.B, self.D, self.core)
        snap = [t.clone() for t in state]

        def run(rows):
            for t, v in zip(state, snap):
                t.copy_(v)
            meta, nch = self.cp_table(rows)
            _lib.call("fh_cp_als", len(self.names), nch, P(meta), P(self.A), P(self.B), P(self.D),
                      P(self.Y), self.ld, self.rp, self.R, self.ld, 1, P(self.core), None,
                      P(self.cp_ws), self.cp_ws.numel(), P(self.status), self.sp())

        sig = (self.nb, len(self.names), self.max_rank, self.R, self.ld)
        dev = self.torch.cuda.get_device_name(self.device)
        rows = autotune.default_tuner().choose(dev, "cp_chunk_rows", sig, [8, 4, 16], run)
        for t, v in zip(state, snap):
            t.copy_(v)
        self.cp_meta, self.nchunks = self.cp_table(rows)

    def cp_als(self, n_iter):
        P = _lib.ptr
        if not self._cp_tuned:
            self.tune_cp()
        self._timed("cp_als", lambda: _lib.call(
            "fh_cp_als", len(self.names), self.nchunks, P(self.cp_meta), P(self.A), P(self.B),
            P(self.D), P(self.Y), self.ld, self.rp, self.R, self.ld, n_iter, P(self.core), None,
            P(self.cp_ws), self.cp_ws.numel(), P(self.status), self.sp()))

    # ------------------------------------------------------------------ ALS
    def update(self, first):
        """update_meta_embedding_interactions (parafac2_intergrative.py:304-540)."""
        if first:
            self.xe()
        self.procrustes()
        self.xg(self.C)
        self.meta_polar(self.C, self.E)
        self.xe()
        self.project_y()

    def iterate(self, first, n_iter_parafac, hist):
        """One fit-loop iteration (parafac2_intergrative.py:635-706); hist receives the loss
        scalars: per-bin-row sum(S), <E, SVD_term^T>, and the core norms before CP-ALS."""
        self.update(first)
        hist["ssum"].copy_(self.ssum)
        hist["meta"].copy_(self.meta_ssum)
        hist["core"].copy_(self.core_ds if self.multi else self.core)
        self.cp_als(n_iter_parafac)
        if self.multi:
            self.dataset_cores()

    @staticmethod
    def parafac_schedule(n_iter, n_iter_parafac):
        """CP-ALS sweeps per fit iteration: one more every 10 iterations, at most 10
        (parafac2_intergrative.py:636-637)."""
        out = []
        for it in range(n_iter):
            if it % 10 == 0 and it > 0 and n_iter_parafac < 10:
                n_iter_parafac += 1
            out.append(n_iter_parafac)
        return out

    def run_iterations(self, n_iter, n_iter_parafac, hist, graph=True):
        """n_iter fit iterations with no host synchronisation.  With graph=True the whole
        sequence is captured once into a CUDA graph (per schedule and history buffers) and
        replayed: every launch, buffer and tensor map in it is fixed, so replays are exact
        repeats of the eager launches.  The capture runs after one eager pass has set every
        kernel's shared-memory attribute.  A budgeted engine starts every sequence with empty
        staging slots (its first pass copies its windows in), so a replay depends on nothing
        an earlier launch left in them; after a replay the slots hold what the captured
        sequence left."""
        torch = self.torch
        sched = self.parafac_schedule(n_iter, n_iter_parafac)
        if self.xs is not None:
            self.xs.reset()
        if not graph:
            for it in range(n_iter):
                self.iterate(it == 0, sched[it], hist[it])
            return
        key = (tuple(sched), tuple(h["ssum"].data_ptr() for h in hist[:n_iter]))
        if key not in getattr(self, "_graphs", {}):
            if not getattr(self, "_warm", False):
                for it in range(n_iter):             # eager pass: attributes, lazy init
                    self.iterate(it == 0, sched[it], hist[it])
                self._warm = True
                return
            g = torch.cuda.CUDAGraph()
            cap = torch.cuda.Stream(device=self.device)
            cap.wait_stream(torch.cuda.current_stream(self.device))
            n0 = _lib.launches
            l0 = self.xs.link_bytes if self.xs is not None else 0
            with torch.cuda.graph(g, stream=cap):
                for it in range(n_iter):
                    self.iterate(it == 0, sched[it], hist[it])
            torch.cuda.current_stream(self.device).wait_stream(cap)
            n_kernels = _lib.launches - n0          # captured, not yet launched
            _lib.launches = n0
            copied = 0
            slots = None
            if self.xs is not None:                 # window copies: captured, not yet run
                copied = self.xs.link_bytes - l0
                self.xs.link_bytes = l0
                slots = list(self.xs.slot_win)
            if not hasattr(self, "_graphs"):
                self._graphs = {}
            self._graphs[key] = (g, n_kernels, slots, copied)
        g, n_kernels, slots, copied = self._graphs[key]
        g.replay()
        if self.xs is not None:
            self.xs.slot_win = list(slots)
            self.xs.link_bytes += copied
        _lib.launches += n_kernels                  # the kernels each replay runs

    def core_norm(self):
        P = _lib.ptr
        _lib.call("fh_core_norm", len(self.names), self.nchunks, P(self.cp_meta), P(self.A),
                  P(self.B), P(self.D), P(self.Y), self.ld, self.rp, self.R, self.ld,
                  P(self.core), P(self.cp_ws), self.cp_ws.numel(), P(self.status), self.sp())
        if self.multi:
            self.dataset_cores()

    def new_history(self, n):
        torch = self.torch
        return [dict(ssum=torch.zeros(self.nb, dtype=torch.float64, device=self.device),
                     meta=torch.zeros(1, dtype=torch.float64, device=self.device),
                     core=torch.zeros(len(self.schic) if self.multi else len(self.names),
                                      dtype=torch.float64, device=self.device))
                for _ in range(n)]

    def losses(self, hist, tnorm):
        """rec_error (total) and per-dataset rec_error of the reference (:667-713)."""
        ssum = hist["ssum"].cpu().numpy()
        core = hist["core"].cpu().numpy()
        xU = np.array([ssum[self.ds_rows[k]].sum() for k in range(len(self.schic))])
        core_ds = core if self.multi else np.array([core[self.chrom_index[k]]
                                                    for k in range(len(self.schic))])
        by_block = tnorm + core_ds - 2 * xU
        rec_V = tnorm.sum() + core_ds.sum() - 2 * float(hist["meta"].item())
        norm_tensor = np.sqrt(tnorm)
        total = math.sqrt(rec_V) / float(np.linalg.norm(norm_tensor)) if rec_V > 0 else float("nan")
        with np.errstate(invalid="ignore"):
            block = np.sqrt(by_block) / norm_tensor
        return total, block

    def transform(self):
        """Final SVD_term over good and bad cells with the stored projections and the
        current factors, and its polar factor (parafac2_intergrative.py:742-834)."""
        P = _lib.ptr
        _lib.call("fh_projection_g_f32", P(self.tiles_dev), P(self.row_tile), self.nb,
                  self.max_width, self.max_rank, P(self.A), self.ld, P(self.B), P(self.D),
                  self.ld, self.R, self.rp, P(self.U), P(self.Gt), self.sp())
        self.xg(self.Ct)
        E_all = self.torch.zeros((self.Ct, self.rp), dtype=self.torch.float32, device=self.device)
        self.meta_polar(self.Ct, E_all)
        return E_all[:, :self.R]
