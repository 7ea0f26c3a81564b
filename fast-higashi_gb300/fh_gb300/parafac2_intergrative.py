"""Fast_Higashi_core on one GB300 (drop-in for fasthigashi.parafac2_intergrative).

Same constructor, ``fit`` / ``transform`` / ``fit_transform`` signatures and the attributes
callers read (A_list, B_dict, D_dict, meta_embedding, projection_list,
projected_tensor_list, n_i, bin_cov_list, chrom2size), computed by the CUDA kernels of
libfhgb300.so.  Factor tensors live on the GPU (the reference keeps A_list and the
projections in pinned host memory); they are torch tensors, so ``.cpu()`` works as before.

Supported options: do_rwr True/False, do_conv True/False (the 3 x 3 mean of
partial_rwr.py:79-83 runs on the fp32 CUDA-core walk in every precision form), do_col
True/False (the column-normalised walk of partial_rwr.py:131-138 on fp32 CUDA cores, with the
coverage rows bin_cov_list / bad_bin_cov_list that init_params computes or the caller
assigns), one or several resolutions (res_list: the datasets of a chromosome share its B and
D, and its CP-ALS runs on their bin rows together, parafac2_intergrative.py:558-590, 674-706),
ranks r <= R <= 128 with at least r compact columns in every bin batch.  Anything else raises
NotImplementedError or FHError.
"""
from __future__ import annotations

import math
import sys
import time

import numpy as np

from . import _lib
from .engine import FitEngine


class Fast_Higashi_core:
    def __init__(self, rank, off_diag, res_list, precision="fp32", hbm_budget=None):
        """precision: "fp32" is the plain drop-in (the reference's arithmetic on CUDA cores);
        "bf16x2" keeps the RWR output as two bf16 planes (16 significant bits) and runs the
        passes over it on the tensor cores; "bf16" keeps one plane (X rounded to bf16).
        hbm_budget: bytes of device memory the fit may hold (None: everything resident); when
        X does not fit, its last chromosomes stream from host memory (fh_gb300/xstream.py) and
        the contact segments are built one dataset at a time."""
        self.rank = rank
        self.precision = precision
        self.hbm_budget = hbm_budget
        self.use_graph = True
        self.sparse_conv = False
        self.off_diag = off_diag
        self.res_list = res_list
        import torch
        self.device = torch.device("cpu")
        self.engine = None
        self.rec_errors_total = []
        self.rec_errors = []

    def to(self, device):
        import torch
        self.device = torch.device(device)
        return self

    # ------------------------------------------------------------------ sizes
    def _sizes(self, schic, size_ratio, size_list):
        """chrom2size and per-dataset bin offsets (parafac2_intergrative.py:558-590)."""
        if size_list is None:
            size_list = [min(int(d.shape[0] * size_ratio * d.resolution / 1000000), self.rank)
                         for d in schic]
            chrom2size = {}
            for d, s in zip(schic, size_list):
                chrom2size[d.chrom] = min(chrom2size.get(d.chrom, s), s)
        else:
            chrom2size = {}
            for d, s in zip(schic, size_list):
                if d.chrom in chrom2size and chrom2size[d.chrom] != s:
                    raise EOFError("size of the same chromosome must be same!")
                chrom2size[d.chrom] = s
        self.chrom2size = chrom2size
        self.chrom2num_bin = {}
        self.chrom2id = {c: [] for c in chrom2size}
        for k, d in enumerate(schic):
            self.chrom2id[d.chrom].append(k)
            if d.chrom not in self.chrom2num_bin:
                self.chrom2num_bin[d.chrom] = d.num_bin
                d.global_slice_bin = slice(0, d.num_bin)
            else:
                d.global_slice_bin = slice(self.chrom2num_bin[d.chrom],
                                           self.chrom2num_bin[d.chrom] + d.num_bin)
                self.chrom2num_bin[d.chrom] += d.num_bin

    # ------------------------------------------------------------------ init
    def init_params(self, schic, do_conv, do_rwr, do_col, seed=None):
        """Initial factors (parafac2_intergrative.py:61-301): A = 1 + 0.01 N(0,1) and
        B = I + 0.01 N (the same draws as the reference from torch's generators), n_i from
        the auto-stop RWR rule evaluated on the GPU, and the meta-embedding / D from a
        randomized SVD of the RWR features computed with the library's X passes."""
        from .init import init_params
        init_params(self, schic, do_conv, do_rwr, do_col, seed=seed)

    # ------------------------------------------------------------------ fit
    def _coverage_src(self):
        return (getattr(self, "bin_cov_list", None), getattr(self, "bad_bin_cov_list", None))

    def _coverage(self):
        """(bin_cov_list, bad_bin_cov_list), or None while no coverage rows are set."""
        good, bad = self._coverage_src()
        if good is None or any(c is None for c in good):
            return None
        return good, (bad if bad is not None else [0] * len(good))

    def _engine(self, schic, do_rwr, do_conv=False, do_col=False):
        col = bool(do_col) and bool(do_rwr)
        if (self.engine is None or self.engine.schic is not schic or
                self.engine.do_conv != bool(do_conv) or self.engine.do_col != col):
            cov = self._coverage() if col else None
            if col and cov is None:
                raise _lib.FHError("fit", 1, "do_col needs bin_cov_list (init_params sets it)")
            self.engine = FitEngine(schic, self.rank, self.chrom2size, self.n_i, self.device,
                                    do_rwr=do_rwr, precision=self.precision, do_conv=do_conv,
                                    do_col=col, bin_cov=cov,
                                    hbm_budget=getattr(self, "hbm_budget", None))
            if col:
                self.engine.cov_src = self._coverage_src()
        elif col:
            src = self._coverage_src()
            held = self.engine.cov_src
            if held is None or held[0] is not src[0] or held[1] is not src[1]:
                # coverage rows assigned since the walk ran: take them and walk again
                cov = self._coverage()
                if cov is None:
                    raise _lib.FHError("fit", 1, "do_col needs bin_cov_list (init_params sets it)")
                self.engine.set_coverage(*cov)
                self.engine.cov_src = src
                self.engine.run_rwr()
        return self.engine

    def fit(self, schic, size_ratio=0.3, n_iter_max=2000, n_iter_parafac=5, do_conv=True,
            do_rwr=False, do_col=False, tol=1e-8, size_list=None, gpu_id=None, verbose=True,
            run_init=True):
        self.gpu_id = gpu_id
        self._sizes(schic, size_ratio, size_list)
        if verbose:
            print("empty params initialized")
        if run_init:
            self.init_params(schic, do_conv, do_rwr, do_col)
        eng = self._engine(schic, do_rwr, do_conv, do_col)
        eng.set_state(self.A_list, self.B_dict, self.D_dict, self.meta_embedding)
        self.tensor_norm = eng.tensor_norms()
        eng.core_norm()
        hist = eng.new_history(n_iter_max)
        self.rec_errors_total, self.rec_errors = [], []
        lines = []
        t_start = time.time()
        done = n_iter_max
        if tol > 0:
            for it in range(n_iter_max):
                if it % 10 == 0 and it > 0 and n_iter_parafac < 10:
                    n_iter_parafac += 1
                eng.iterate(it == 0, n_iter_parafac, hist[it])
                # _record reads the loss scalars (a device round trip each iteration), so a
                # kernel error stops the fit here instead of running on NaN losses
                eng.check_status("fit")
                if self._record(eng, hist[it], it, lines, verbose, t_start, tol):
                    done = it + 1
                    break
        else:
            # no stopping rule: the iterations need no host round trip and run as one CUDA
            # graph once the engine has run them eagerly
            eng.run_iterations(n_iter_max, n_iter_parafac, hist, graph=self.use_graph)
            for it in range(n_iter_max):
                self._record(eng, hist[it], it, lines, verbose, t_start, tol)
        eng.check_status("fit")
        self.n_iter_done = done
        self._publish(eng)
        return self

    def _record(self, eng, h, it, lines, verbose, t_start, tol):
        total, block = eng.losses(h, self.tensor_norm)
        self.rec_errors_total.append(total)
        self.rec_errors.append(block)
        stop = False
        if it >= 1:
            r = self.rec_errors
            t = self.rec_errors_total
            diff = (r[-2] ** 2 - r[-1] ** 2) / r[-2] ** 2
            tdiff = (t[-2] ** 2 - t[-1] ** 2) / t[-2] ** 2
            msg = ("PARAFAC2 re=%.3f %.2e variation min%.1e at chrom %d, max%.1e at chrom %d"
                   % (total, tdiff, diff.min(), diff.argmin(), diff.max(), diff.argmax()))
            stop = it >= 3 and tol > 0 and (tdiff < tol or diff.max() < tol * 2)
        else:
            msg = "PARAFAC2 re=%.3f" % total
        if verbose:
            print(msg, "takes %.1fs" % (time.time() - t_start))
            if stop:
                print("converged in {} iterations.".format(it))
            sys.stdout.flush()
        lines.append(msg)
        return stop

    def _publish(self, eng):
        self.A_list = eng.A_views()
        self.B_dict = eng.B_views()
        self.D_dict = eng.D_views()
        self.meta_embedding = eng.E[:, :self.rank]
        self.projection_list = eng.projection_views()
        self.projected_tensor_list = eng.projected_views()

    def update_meta_embedding_interactions(self, schic, projection_list=None,
                                           projected_tensor_list=None, do_conv=True, do_rwr=True,
                                           do_col=False, first_iter=False):
        """One update (parafac2_intergrative.py:304-540) from the current state.  Returns
        (projection_list, projected_tensor_list, rec_error_x_U, rec_error_x_V
        [, rec_error_tensor_norm])."""
        eng = self._engine(schic, do_rwr, do_conv, do_col)
        eng.set_state(self.A_list, self.B_dict, self.D_dict, self.meta_embedding)
        eng.update(first=True)
        eng.check_status("update_meta_embedding_interactions")
        ssum = eng.ssum.cpu().numpy()
        xU = np.array([[ssum[eng.ds_rows[k]].sum()] for k in range(len(schic))])
        xV = float(eng.meta_ssum.item())
        self.meta_embedding = eng.E[:, :self.rank]
        out = (eng.projection_views(), eng.projected_views(), xU, xV)
        if first_iter:
            return out + (eng.tensor_norms().reshape(-1, 1),)
        return out

    # ------------------------------------------------------------------ transform
    def transform(self, schic, do_conv, do_rwr, do_col):
        eng = self._engine(schic, do_rwr, do_conv, do_col)
        E = eng.transform()
        eng.check_status("transform")
        return (None, (self.A_list, self.B_dict.values(), self.D_dict.values(), E),
                self.projection_list)

    def fit_transform(self, schic, size_ratio=0.3, n_iter_max=2000, n_iter_parafac=5,
                      do_conv=True, do_rwr=False, do_col=False, tol=1e-8, size_list=None,
                      gpu_id=None, verbose=True, run_init=True):
        if verbose:
            print("n_iter_parafac", n_iter_parafac)
        self.fit(schic, size_ratio, n_iter_max, n_iter_parafac, do_conv, do_rwr, do_col, tol,
                 size_list, gpu_id, verbose, run_init)
        return self.transform(schic, do_conv, do_rwr, do_col)
