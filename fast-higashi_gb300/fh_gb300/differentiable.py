"""The fit's reconstruction loss as a differentiable layer (a torch.autograd.Function).

The model reconstructs bin batch i of a chromosome as X_i[:, :, c] ~ U_i lhs_i[c]^T with
lhs_i[c][l] = sum_p A[i, p] B[l, p] (E D)[c, p] (parafac2_intergrative.py:336-383; its
reconstruction error is :667-713).  Split by cell, the loss is

    L_c(rp, E, A, B, D) = sum over chromosomes, bin rows i and band columns j of
                          (X_i(rp)[j, c] - sum_l U_i[j, l] lhs_i[c][l])^2

with X(rp) the partial RWR output for the walk weight rp of partial_rwr.py:109,116-118
(Q_{t+1} = rp Q_t P + (1 - rp) I; the fit uses 0.5) and U the bin rows' projections, held
fixed (the fit's last Procrustes step).  Gradients flow to rp, E (cells x R) and every
chromosome's A (bins x r), B (r x r) and D (R x r).

Forward: the RWR at rp (fh_rwr_tiles_rp_f32), the rows Gt = U B diag(A) D^T
(fh_projection_g_f32), the fused per-cell loss (fh_recon_loss_f32); X is not kept.
Backward: X and dX/drp recomputed tile by tile (fh_rwr_grad_f32), the fused residual
backward (fh_recon_loss_bwd_f32: dE, dGt, drp), H = U^T dGt (fh_project_y_f32) and the
factor gradients (fh_factor_grad_f32).  fp32 arithmetic, fp64 loss sums; all on the GPU.

    layer = ReconstructionLoss(model)          # a fitted Fast_Higashi_core
    loss = layer(rp, E, A_list, B_list, D_list)  # (cells,) float64
    loss.sum().backward()
"""
from __future__ import annotations

import torch

from . import _lib


class ReconstructionLoss:
    """Per-cell reconstruction loss over a fitted model's contacts and projections.

    model: a fitted Fast_Higashi_core (or its FitEngine).  Factor lists follow the datasets'
    order (A_list, B_dict.values(), D_dict.values() of the model)."""

    def __init__(self, model):
        eng = getattr(model, "engine", model)
        if eng is None or not hasattr(eng, "tiles_dev"):
            raise _lib.FHError("ReconstructionLoss", 1, "the model has not been fitted")
        if eng.max_rank > 64 or eng.rp > 64:
            raise _lib.FHError("ReconstructionLoss", 2, "ranks above 64 are not supported")
        if eng.do_conv or eng.do_col:
            raise _lib.FHError("ReconstructionLoss", 2,
                               "the differentiable walk covers do_conv=False, do_col=False")
        if getattr(eng, "xs", None) is not None:
            raise _lib.FHError("ReconstructionLoss", 2,
                               "the differentiable walk needs X resident (no hbm_budget)")
        self.eng = eng
        self.torch = torch
        self._ws = {}
        self.timing = None   # {step: [(start event, end event)]} when enabled

    def __call__(self, rp, E, A_list, B_list, D_list):
        torch = self.torch
        if not torch.is_tensor(rp):
            rp = torch.tensor(float(rp), dtype=torch.float64, device=self.eng.device)
        n = len(self.eng.schic)
        if not (len(A_list) == len(B_list) == len(D_list) == n):
            raise _lib.FHError("ReconstructionLoss", 1, "one A, B and D per dataset")
        return ReconFn.apply(self, rp, E, *A_list, *B_list, *D_list)

    # ------------------------------------------------------------------ helpers
    def _timed(self, name, fn):
        """Runs fn; with timing enabled, brackets it with CUDA events on the current stream."""
        if self.timing is None:
            return fn()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        out = fn()
        e.record()
        self.timing.setdefault(name, []).append((s, e))
        return out

    def timing_summary(self):
        return {k: {"launches": len(v), "total_ms": sum(a.elapsed_time(b) for a, b in v),
                    "mean_ms": sum(a.elapsed_time(b) for a, b in v) / len(v)}
                for k, v in (self.timing or {}).items()}

    def _buf(self, key, nbytes):
        t = self._ws.get(key)
        if t is None or t.numel() < nbytes:
            t = self.torch.empty(max(int(nbytes), 1), dtype=self.torch.uint8, device=self.eng.device)
            self._ws[key] = t
        return t

    def pack(self, E, A_list, B_list, D_list):
        """Factors in the engine's padded layouts (copies; the fit state is not touched)."""
        torch, eng = self.torch, self.eng
        f32, dev = torch.float32, eng.device
        nchrom = len(eng.names)
        Ep = torch.zeros((eng.C, eng.rp), dtype=f32, device=dev)
        Ep[:, :eng.R] = E.detach().to(dev, f32)
        Ap = torch.zeros((eng.nb, eng.ld), dtype=f32, device=dev)
        Bp = torch.zeros((nchrom, eng.ld, eng.ld), dtype=f32, device=dev)
        Dp = torch.zeros((nchrom, eng.rp, eng.ld), dtype=f32, device=dev)
        for k in range(len(eng.schic)):
            r, ci = eng.ranks[k], eng.chrom_index[k]
            Ap[eng.ds_rows[k], :r] = A_list[k].detach().to(dev, f32)
            Bp[ci, :r, :r] = B_list[k].detach().to(dev, f32)
            Dp[ci, :eng.R, :r] = D_list[k].detach().to(dev, f32)
        return Ep, Ap, Bp, Dp

    def rwr(self, rp, grad=False):
        """X (and dX/drp with grad=True) for all cells at walk weight rp."""
        torch, eng = self.torch, self.eng
        P = _lib.ptr
        X = torch.empty((eng.Ct, eng.ldx), dtype=torch.float32, device=eng.device)
        if grad:
            Xp = torch.empty_like(X)
            self._timed("rwr_grad", lambda: _lib.call(
                "fh_rwr_grad_f32", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
                eng.max_width, P(eng.store.entries), P(eng.store.offsets), rp, P(X), P(Xp),
                eng.ldx, P(eng.status), _lib.stream_ptr()))
            return X, Xp
        self._timed("rwr_rp", lambda: _lib.call(
            "fh_rwr_tiles_rp_f32", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
            eng.max_width, P(eng.store.entries), P(eng.store.offsets), rp, P(X), eng.ldx, None,
            P(eng.status), _lib.stream_ptr()))
        return X

    def gt(self, Ap, Bp, Dp):
        torch, eng = self.torch, self.eng
        Gt = torch.empty((eng.rows, eng.rp), dtype=torch.float32, device=eng.device)
        P = _lib.ptr
        self._timed("projection_g", lambda: _lib.call(
            "fh_projection_g_f32", P(eng.tiles_dev), P(eng.row_tile), eng.nb, eng.max_width,
            eng.max_rank, P(Ap), eng.ld, P(Bp), P(Dp), eng.ld, eng.R, eng.rp, P(eng.U), P(Gt),
            _lib.stream_ptr()))
        return Gt

    def recon_ws(self):
        eng = self.eng
        n = _lib.value("fh_recon_workspace", eng.C, eng.rows, eng.rp)
        return self._buf("recon", n), n


def _as(t, meta):
    return t.to(dtype=meta[0], device=meta[1])


class ReconFn(torch.autograd.Function):
    """forward(op, rp, E, *A_list, *B_list, *D_list) -> per-cell loss (float64)."""

    @staticmethod
    def forward(ctx, op, rp, E, *fs):
        eng = op.eng
        n = len(eng.schic)
        P = _lib.ptr
        rpv = float(rp)
        Ep, Ap, Bp, Dp = op.pack(E, fs[:n], fs[n:2 * n], fs[2 * n:])
        X = op.rwr(rpv)
        Gt = op.gt(Ap, Bp, Dp)
        loss = torch.empty(eng.C, dtype=torch.float64, device=eng.device)
        ws, nbytes = op.recon_ws()
        op._timed("recon_loss", lambda: _lib.call(
            "fh_recon_loss_f32", P(X), eng.ldx, eng.C, eng.rows, P(Gt), P(Ep), eng.rp, P(loss),
            P(ws), nbytes, _lib.stream_ptr()))
        del X
        eng.check_status("ReconstructionLoss.forward")
        ctx.op, ctx.rpv, ctx.n = op, rpv, n
        ctx.in_meta = [(t.dtype, t.device) for t in (rp, E) + tuple(fs)]
        ctx.save_for_backward(Ep, Ap, Bp, Dp, Gt)
        return loss

    @staticmethod
    def backward(ctx, g):
        op, n = ctx.op, ctx.n
        eng = op.eng
        Ep, Ap, Bp, Dp, Gt = ctx.saved_tensors
        P = _lib.ptr
        sp = _lib.stream_ptr()
        w = g.detach().to(eng.device, torch.float64).contiguous()
        X, Xp = op.rwr(ctx.rpv, grad=True)
        dE = torch.empty_like(Ep)
        dGt = torch.empty_like(Gt)
        drp = torch.empty(1, dtype=torch.float64, device=eng.device)
        ws, nbytes = op.recon_ws()
        op._timed("recon_bwd", lambda: _lib.call(
            "fh_recon_loss_bwd_f32", P(X), P(Xp), eng.ldx, eng.C, eng.rows, P(Gt), P(Ep), eng.rp,
            P(w), None, P(dE), P(dGt), P(drp), P(ws), nbytes, sp))
        del X, Xp
        H = torch.empty((eng.nb, eng.ld, eng.rp), dtype=torch.float32, device=eng.device)
        op._timed("project_h", lambda: _lib.call(
            "fh_project_y_f32", P(eng.tiles_dev), P(eng.row_tile), eng.nb, P(eng.U), P(dGt),
            eng.rp, P(H), eng.ld, sp))
        dA, dB, dD = torch.empty_like(Ap), torch.empty_like(Bp), torch.empty_like(Dp)
        fw = _lib.value("fh_factor_grad_workspace", eng.nchunks, eng.ld, eng.rp)
        fws = op._buf("factor", fw)
        op._timed("factor_grad", lambda: _lib.call(
            "fh_factor_grad_f32", len(eng.names), eng.nchunks, P(eng.cp_meta), P(H), eng.ld,
            P(Ap), P(Bp), P(Dp), eng.ld, eng.rp, eng.R, P(dA), P(dB), P(dD), P(fws), fw, sp))
        eng.check_status("ReconstructionLoss.backward")
        meta = ctx.in_meta
        out = [None, _as(drp.reshape(()), meta[0]), _as(dE[:, :eng.R], meta[1])]
        for k in range(n):
            out.append(_as(dA[eng.ds_rows[k], :eng.ranks[k]], meta[2 + k]))
        for k in range(n):
            r, ci = eng.ranks[k], eng.chrom_index[k]
            out.append(_as(dB[ci, :r, :r], meta[2 + n + k]))
        for k in range(n):
            r, ci = eng.ranks[k], eng.chrom_index[k]
            out.append(_as(dD[ci, :eng.R, :r], meta[2 + 2 * n + k]))
        return tuple(out)
