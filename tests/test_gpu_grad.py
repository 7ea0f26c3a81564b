"""GPU checks of the differentiable reconstruction loss (fh_gb300.differentiable).

The loss (per cell c, over every chromosome's bin batches i and band columns j):
    L_c = sum (X_i(rp)[c, :, :] - recon_i[:, c, :])^2,
    recon_i[j, c] = U_i[j] lhs_i[c],  lhs = KR(A_i, B, E D)   (parafac2_intergrative.py:336-383)
with X(rp) the partial RWR of partial_rwr.py:84-138 at walk weight rp (0.5 in the fit).

Checks and tolerances (relative Frobenius error unless stated):
  fh_rwr_tiles_rp_f32 at rp = 0.5    bit-identical to the fit's fh_rwr_tiles_f32
  fh_rwr_grad_f32                    X bit-identical to fh_rwr_tiles_rp_f32; dX/drp within
                                     1e-5 of an fp64 central difference (h = 1e-5) of the
                                     restated RWR
  small fit, random cell weights     loss within 1e-6 of torch autograd of the reference
                                     formula in float64 on the same contacts, projections and
                                     factors; every gradient (rp, E, A, B, D) within 1e-5 of
                                     its scale (below)
  2,000 cells at 500 kb (R = 32,     central differences (h = 1e-3) of the float64 loss on 64
  band 20, fp32)                     random coordinates (rp, E, A, B, D):
                                     |g - fd| <= 1e-5 * scale of that coordinate
A gradient of this loss is a sum of many terms of both signs (dE[c] = -2 sum_rows Res[c] Gt,
and near a fitted state Res is nearly orthogonal to Gt), so its fp32 error is bounded by the
size of its terms, not by its value: the scale of a coordinate is the same gradient formula
evaluated on absolute values (sum of |w| |Res| |Gt| for E, and so on through the chain).
fp32 inputs (the RWR output X itself is fp32) leave errors of about 1e-6 of that scale.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib
import fp64_reference as F
import golden_io as G
from gpu_util import datasets_from

pytestmark = pytest.mark.gpu

CUDA = torch.device("cuda")
F64 = torch.float64
P = _lib.ptr


def sp():
    return _lib.stream_ptr()


def rel(a, b):
    a, b = a.double(), b.double()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b).clamp_min(1e-300))


def golden_engine():
    from fh_gb300.engine import FitEngine
    z = G.load("rwr_tiles.npz")
    ds = datasets_from(z, resolution=1000000)
    return FitEngine(ds, 4, {d.chrom: 2 for d in ds}, [3] * len(ds), CUDA)


def rwr_rp(eng, rp):
    X = torch.full((eng.Ct, eng.ldx), float("nan"), device=CUDA)
    _lib.call("fh_rwr_tiles_rp_f32", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
              eng.max_width, P(eng.store.entries), P(eng.store.offsets), rp, P(X), eng.ldx,
              None, P(eng.status), sp())
    return X


def test_rwr_rp_half_is_the_fit_rwr():
    eng = golden_engine()
    X = rwr_rp(eng, 0.5)
    torch.cuda.synchronize()
    assert torch.equal(X[:, :eng.rows], eng.X[:, :eng.rows])


def _fit_small(name, iters, seed=0):
    """A short fp32 fit of a synthetic workload; returns (model, oracle ChromData list)."""
    from fh_gb300 import Fast_Higashi_core, synth
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    w = synth.workload(name)
    coo, _ = synth.generate(w, seed=seed)
    ds, bsb, bsc = [], [], []
    for (idx, val, shape), cname, nb in zip(coo, w.chrom_names, w.chrom_bins):
        b, c = synth.recommend_batches(w, nb, w.n_cells)
        bsb.append(b)
        bsc.append(c)
        ds.append(Chrom_Dataset(Sparse(idx, val, shape, copy=False), b, c, compact=True,
                                flank=w.band, chrom=cname, resolution=w.resolution))
    datas = F.chrom_datas(coo, w.chrom_names, bsb, bsc, w.band)
    torch.manual_seed(seed)
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution]).to(CUDA)
    m.fit(ds, size_ratio=w.dim1, n_iter_max=iters, n_iter_parafac=1, do_conv=False,
          do_rwr=True, do_col=False, tol=0, verbose=False)
    torch.cuda.synchronize()
    return m, ds, datas


def test_rwr_grad_matches_forward_and_fp64_difference():
    m, ds, datas = _fit_small("small", 1)
    eng = m.engine
    rp = 0.3
    X = torch.empty((eng.Ct, eng.ldx), device=CUDA)
    Xp = torch.empty_like(X)
    _lib.call("fh_rwr_grad_f32", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
              eng.max_width, P(eng.store.entries), P(eng.store.offsets), rp, P(X), P(Xp), eng.ldx,
              P(eng.status), sp())
    X0 = rwr_rp(eng, rp)
    torch.cuda.synchronize()
    eng.check_status("rwr_grad")
    assert torch.equal(X[:, :eng.rows], X0[:, :eng.rows])
    h = 1e-5
    ref = torch.empty((eng.Ct, eng.rows), dtype=F64, device=CUDA)
    off = 0
    for ci, bi, bb, A in F.dense_tiles(datas, eng.Ct, CUDA):
        n_i = int(eng.n_rwr[ci])
        d = (F.rwr_tile(A, bb.local.start, bb.local.stop, n_i, rp + h)
             - F.rwr_tile(A, bb.local.start, bb.local.stop, n_i, rp - h)) / (2 * h)
        ref[:, off:off + bb.rows * bb.width] = d.reshape(eng.Ct, -1)
        off += bb.rows * bb.width
    assert off == eng.rows
    assert rel(Xp[:, :eng.rows], ref) < 1e-5


def _gt_rows(U, A_blk, B, D):
    """Gt rows of a bin batch: U_i B diag(A_i) D^T -> (b, n, R)."""
    return torch.einsum("ijl,lp,ip,mp->ijm", U, B, A_blk, D)


def _tile_scales(X, U, A_blk, Bc, Dc, E, w):
    """Residual of a bin batch and the absolute-value scales of its gradient terms."""
    Gt = _gt_rows(U, A_blk, Bc, Dc)
    Res = X - torch.einsum("ijm,km->kij", Gt, E)
    aR = Res.abs() * w.abs()[:, None, None]
    sE = 2 * torch.einsum("kij,ijm->km", aR, Gt.abs())
    sGt = 2 * torch.einsum("kij,km->ijm", aR, E.abs())
    Habs = torch.einsum("ijl,ijm->ilm", U.abs(), sGt)
    Tabs = torch.einsum("ilm,mp->ilp", Habs, Dc.abs())
    sA = torch.einsum("lp,ilp->ip", Bc.abs(), Tabs)
    sB = torch.einsum("ip,ilp->lp", A_blk.abs(), Tabs)
    sD = torch.einsum("ilm,lp,ip->mp", Habs, Bc.abs(), A_blk.abs())
    return Res, sE, sA, sB, sD


class _Scales:
    """Gradient scales summed over bin batches (per-dataset A, B, D)."""

    def __init__(self, A64, B64, D64, E64):
        self.sE = torch.zeros_like(E64)
        self.sA = [torch.zeros_like(a) for a in A64]
        self.sB = [torch.zeros_like(b) for b in B64]
        self.sD = [torch.zeros_like(d) for d in D64]
        self.srp = 0.0

    def add(self, ci, bb, X, U, A64, B64, D64, E64, w):
        Res, sE, sA, sB, sD = _tile_scales(X, U, A64[ci][bb.start:bb.start + bb.rows], B64[ci],
                                           D64[ci], E64, w)
        self.sE += sE
        self.sA[ci][bb.start:bb.start + bb.rows] += sA
        self.sB[ci] += sB
        self.sD[ci] += sD
        return Res


def _reference_loss(datas, views, n_rwr, C, rp, E, A_list, B_list, D_list):
    """The loss restated from the reference's formulas in float64 torch (autograd-able)."""
    out = torch.zeros(C, dtype=F64, device=CUDA)
    for ci, bi, bb, Ad in F.dense_tiles(datas, C, CUDA):
        X = F.rwr_tile(Ad, bb.local.start, bb.local.stop, int(n_rwr[ci]), rp)  # (C, b, n)
        U = views[ci][bi].double()                                             # (b, n, r)
        A_blk = A_list[ci][bb.start:bb.start + bb.rows]
        lhs = torch.einsum("ir,jr,kr->ikj", A_blk, B_list[ci], E @ D_list[ci])  # (b, C, r)
        recon = torch.einsum("ijl,ikl->kij", U, lhs)                            # (C, b, n)
        out = out + ((X - recon) ** 2).sum((1, 2))
    return out


def _state(m):
    eng = m.engine
    A = [a.detach().clone() for a in m.A_list]
    B = [m.B_dict[d.chrom].detach().clone() for d in eng.schic]
    D = [m.D_dict[d.chrom].detach().clone() for d in eng.schic]
    E = m.meta_embedding.detach().clone()
    return A, B, D, E


def test_recon_loss_matches_torch_autograd_of_reference_formula():
    from fh_gb300.differentiable import ReconstructionLoss
    m, ds, datas = _fit_small("small", 3)
    eng = m.engine
    A, B, D, E = _state(m)
    w = torch.rand(eng.C, dtype=F64, device=CUDA, generator=torch.Generator(CUDA).manual_seed(3))
    # ours (fp32 kernels)
    rp = torch.tensor(0.5, dtype=F64, device=CUDA, requires_grad=True)
    leaves = [E.requires_grad_()] + [t.requires_grad_() for t in A + B + D]
    layer = ReconstructionLoss(m)
    loss = layer(rp, E, A, B, D)
    (loss * w).sum().backward()
    ours = [rp.grad] + [t.grad for t in leaves]
    # torch autograd of the reference formula, float64
    rp64 = torch.tensor(0.5, dtype=F64, device=CUDA, requires_grad=True)
    l64 = [t.detach().double().requires_grad_() for t in leaves]
    n = len(A)
    E64, A64, B64, D64 = l64[0], l64[1:1 + n], l64[1 + n:1 + 2 * n], l64[1 + 2 * n:]
    ref = _reference_loss(datas, eng.projection_views(), eng.n_rwr, eng.C, rp64, E64, A64, B64,
                          D64)
    (ref * w).sum().backward()
    assert rel(loss, ref) < 1e-6
    # scales of the gradient terms (float64, absolute values)
    views = eng.projection_views()
    with torch.no_grad():
        d64 = [t.detach() for t in l64]
        sc = _Scales(d64[1:1 + n], d64[1 + n:1 + 2 * n], d64[1 + 2 * n:], d64[0])
        h = 1e-5
        for ci, bi, bb, Ad in F.dense_tiles(datas, eng.C, CUDA):
            ni = int(eng.n_rwr[ci])
            X = F.rwr_tile(Ad, bb.local.start, bb.local.stop, ni, 0.5)
            Res = sc.add(ci, bb, X, views[ci][bi].double(), d64[1:1 + n], d64[1 + n:1 + 2 * n],
                         d64[1 + 2 * n:], d64[0], w)
            Xp = (F.rwr_tile(Ad, bb.local.start, bb.local.stop, ni, 0.5 + h)
                  - F.rwr_tile(Ad, bb.local.start, bb.local.stop, ni, 0.5 - h)) / (2 * h)
            sc.srp += float(2 * (Res.abs() * Xp.abs() * w.abs()[:, None, None]).sum())
    scales = [torch.tensor(sc.srp, dtype=F64), sc.sE] + sc.sA + sc.sB + sc.sD
    refs = [rp64.grad] + [t.grad for t in l64]
    names = ["rp", "E"] + ["A%d" % k for k in range(n)] + ["B%d" % k for k in range(n)] + \
        ["D%d" % k for k in range(n)]
    errs, plain = {}, {}
    for nm, g, r, s_ in zip(names, ours, refs, scales):
        d = (g.double().cpu() - r.double().cpu()).reshape(-1)
        errs[nm] = float(torch.linalg.norm(d) / torch.linalg.norm(s_.double().cpu().reshape(-1)))
        plain[nm] = float(torch.linalg.norm(d) / torch.linalg.norm(r.double().cpu().reshape(-1)))
    print("scaled gradient errors", errs)
    print("relative gradient errors", plain)
    assert max(errs.values()) < 1e-5, errs


def test_recon_grad_central_differences_2000_cells():
    """2,000 cells at 500 kb, R = 32, band 20: 64 random coordinates."""
    from fh_gb300.differentiable import ReconstructionLoss
    m, ds, datas = _fit_small("c4", 3)
    eng = m.engine
    A, B, D, E = _state(m)
    n = len(A)
    rp = torch.tensor(0.5, dtype=F64, device=CUDA, requires_grad=True)
    leaves = [E.requires_grad_()] + [t.requires_grad_() for t in A + B + D]
    layer = ReconstructionLoss(m)
    loss = layer(rp, E, A, B, D)
    loss.sum().backward()
    gE = E.grad.double()
    gA = [t.grad.double() for t in A]
    gB = [t.grad.double() for t in B]
    gD = [t.grad.double() for t in D]
    g_rp = float(rp.grad)

    # float64 state, cached tiles, the loss and the gradient scales
    views = eng.projection_views()
    E64 = E.detach().double()
    A64 = [t.detach().double() for t in A]
    B64 = [t.detach().double() for t in B]
    D64 = [t.detach().double() for t in D]
    ones = torch.ones(eng.C, dtype=F64, device=CUDA)
    sc = _Scales(A64, B64, D64, E64)
    tiles = {}
    L64 = torch.zeros(eng.C, dtype=F64, device=CUDA)
    for ci, bi, bb, Ad in F.dense_tiles(datas, eng.C, CUDA):
        X = F.rwr_tile(Ad, bb.local.start, bb.local.stop, int(eng.n_rwr[ci]), 0.5)
        U = views[ci][bi].double()
        tiles[(ci, bi)] = (bb, Ad, X, U)
        Res = sc.add(ci, bb, X, U, A64, B64, D64, E64, ones)
        L64 += (Res ** 2).sum((1, 2))
    assert rel(loss.detach(), L64) < 1e-5

    def tile_loss(key, Ev, Av, Bv, Dv, rows=None, cells=None):
        bb, _, X, U = tiles[key]
        Ab = Av[bb.start:bb.start + bb.rows]
        if rows is not None:
            U, Ab, X = U[rows:rows + 1], Ab[rows:rows + 1], X[:, rows:rows + 1]
        if cells is not None:
            X, Ev = X[cells:cells + 1], Ev[cells:cells + 1]
        Gt = _gt_rows(U, Ab, Bv, Dv)
        return float(((X - torch.einsum("ijm,km->kij", Gt, Ev)) ** 2).sum())

    h = 1e-3
    rng = np.random.default_rng(11)
    checks = []   # (name, kernel gradient, central difference, scale)
    # rp: the whole loss at rp +- h (the RWR is recomputed)
    Lpm, Xpm = [0.0, 0.0], {}
    for si, s in enumerate((1, -1)):
        for key, (bb, Ad, X0, U) in tiles.items():
            ci = key[0]
            X = F.rwr_tile(Ad, bb.local.start, bb.local.stop, int(eng.n_rwr[ci]), 0.5 + s * h)
            Gt = _gt_rows(U, A64[ci][bb.start:bb.start + bb.rows], B64[ci], D64[ci])
            Res = X0 - torch.einsum("ijm,km->kij", Gt, E64)
            Lpm[si] += float(((X - X0 + Res) ** 2).sum())
            if s == 1:
                Xpm[key] = X
            else:
                sc.srp += float(2 * (Res.abs() * ((Xpm.pop(key) - X) / (2 * h)).abs()).sum())
    checks.append(("rp", g_rp, (Lpm[0] - Lpm[1]) / (2 * h), sc.srp))
    keys_of = {ci: [k for k in tiles if k[0] == ci] for ci in range(n)}
    for _ in range(21):                                   # E[c, m]: one cell
        c, mm = int(rng.integers(eng.C)), int(rng.integers(eng.R))
        d = 0.0
        for s in (1, -1):
            Ev = E64.clone()
            Ev[c, mm] += s * h
            d += s * sum(tile_loss(k, Ev, A64[k[0]], B64[k[0]], D64[k[0]], cells=c) for k in tiles)
        checks.append(("E[%d,%d]" % (c, mm), float(gE[c, mm]), d / (2 * h), float(sc.sE[c, mm])))
    for _ in range(14):                                   # A[i, p]: one bin row
        k = int(rng.integers(n))
        i, p = int(rng.integers(A64[k].shape[0])), int(rng.integers(A64[k].shape[1]))
        key = next(kk for kk in keys_of[k]
                   if tiles[kk][0].start <= i < tiles[kk][0].start + tiles[kk][0].rows)
        d = 0.0
        for s in (1, -1):
            Av = A64[k].clone()
            Av[i, p] += s * h
            d += s * tile_loss(key, E64, Av, B64[k], D64[k], rows=i - tiles[key][0].start)
        checks.append(("A%d[%d,%d]" % (k, i, p), float(gA[k][i, p]), d / (2 * h),
                       float(sc.sA[k][i, p])))
    for blk, src, grads, scl in (("B", B64, gB, sc.sB), ("D", D64, gD, sc.sD)):
        for _ in range(14):                               # B / D entries: one chromosome
            k = int(rng.integers(n))
            i, p = int(rng.integers(src[k].shape[0])), int(rng.integers(src[k].shape[1]))
            d = 0.0
            for s in (1, -1):
                v = src[k].clone()
                v[i, p] += s * h
                Bv, Dv = (v, D64[k]) if blk == "B" else (B64[k], v)
                d += s * sum(tile_loss(kk, E64, A64[k], Bv, Dv) for kk in keys_of[k])
            checks.append(("%s%d[%d,%d]" % (blk, k, i, p), float(grads[k][i, p]), d / (2 * h),
                           float(scl[k][i, p])))
    assert len(checks) == 64
    worst, worst_rel = 0.0, 0.0
    for name, g, fd, scale in checks:
        err = abs(g - fd) / scale
        worst = max(worst, err)
        worst_rel = max(worst_rel, abs(g - fd) / max(abs(fd), 1e-300))
        print("%-14s kernel %+.6e  central difference %+.6e  scaled error %.1e" % (name, g, fd, err))
    print("central differences: 64 coordinates, worst scaled error %.2e, worst relative %.2e"
          % (worst, worst_rel))
    for name, g, fd, scale in checks:
        assert abs(g - fd) <= 1e-5 * scale, (name, g, fd, scale)
    assert math.isfinite(worst)


@pytest.mark.parametrize("rp,C,rows", [(16, 70, 1013), (32, 64, 4096), (64, 129, 777)])
def test_recon_kernels_on_ragged_shapes(rp, C, rows):
    """fh_recon_loss_f32 / fh_recon_loss_bwd_f32 against float64 torch on random inputs whose
    cells and band rows are not multiples of the 64 x 64 tile (padding past `rows` is NaN)."""
    g = torch.Generator(device="cpu").manual_seed(rp + C)
    ldx = ((rows + 127) // 128) * 128
    X = torch.full((C, ldx), float("nan"))
    X[:, :rows] = torch.rand((C, rows), generator=g)
    Xp = torch.full((C, ldx), float("nan"))
    Xp[:, :rows] = torch.randn((C, rows), generator=g)
    Gt = torch.randn((rows, rp), generator=g) * 0.1
    E = torch.randn((C, rp), generator=g) * 0.1
    w = torch.rand(C, dtype=F64, generator=g)
    X, Xp, Gt, E, w = (t.to(CUDA) for t in (X, Xp, Gt, E, w))
    nbytes = _lib.value("fh_recon_workspace", C, rows, rp)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=CUDA)
    loss = torch.empty(C, dtype=F64, device=CUDA)
    _lib.call("fh_recon_loss_f32", P(X), ldx, C, rows, P(Gt), P(E), rp, P(loss), P(ws), nbytes, sp())
    dE = torch.empty((C, rp), device=CUDA)
    dGt = torch.empty((rows, rp), device=CUDA)
    drp = torch.empty(1, dtype=F64, device=CUDA)
    loss2 = torch.empty(C, dtype=F64, device=CUDA)
    _lib.call("fh_recon_loss_bwd_f32", P(X), P(Xp), ldx, C, rows, P(Gt), P(E), rp, P(w), P(loss2),
              P(dE), P(dGt), P(drp), P(ws), nbytes, sp())
    torch.cuda.synchronize()
    X64, Xp64 = X[:, :rows].double(), Xp[:, :rows].double()
    Res = X64 - E.double() @ Gt.double().T
    assert rel(loss, (Res ** 2).sum(1)) < 1e-6
    assert torch.equal(loss, loss2)
    assert rel(dE, -2 * w[:, None] * (Res @ Gt.double())) < 1e-5
    assert rel(dGt, -2 * (Res * w[:, None]).T @ E.double()) < 1e-5
    ref = 2 * (w * (Res * Xp64).sum(1)).sum()
    assert abs(float(drp) - float(ref)) <= 1e-5 * float(2 * (w * (Res.abs() * Xp64.abs()).sum(1)).sum())


def test_rwr_grad_zero_epochs_and_zero_walk_weight():
    """With no epochs X = A and dX/drp = 0; with rp = 0 one epoch gives X = A and
    dX/drp = P A - A."""
    from fh_gb300.engine import FitEngine
    z = G.load("rwr_tiles.npz")
    ds = datasets_from(z, resolution=1000000)
    for epochs in (0, 1):
        eng = FitEngine(ds, 4, {d.chrom: 2 for d in ds}, [epochs] * len(ds), CUDA)
        X = torch.empty((eng.Ct, eng.ldx), device=CUDA)
        Xp = torch.empty_like(X)
        rp = 0.0 if epochs else 0.5
        _lib.call("fh_rwr_grad_f32", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
                  eng.max_width, P(eng.store.entries), P(eng.store.offsets), rp, P(X), P(Xp),
                  eng.ldx, P(eng.status), sp())
        X0 = rwr_rp(eng, 0.0) if epochs else eng.X
        torch.cuda.synchronize()
        eng.check_status("rwr_grad")
        assert torch.equal(X[:, :eng.rows], X0[:, :eng.rows])
        if epochs == 0:
            assert float(Xp[:, :eng.rows].abs().max()) == 0.0
        else:
            # dX/drp at rp = 0 after one epoch: P A - A = (X(rp) - A) / rp for any rp (linear)
            Xh = rwr_rp(eng, 0.25)
            torch.cuda.synchronize()
            ref = (Xh[:, :eng.rows].double() - X0[:, :eng.rows].double()) / 0.25
            assert rel(Xp[:, :eng.rows], ref) < 1e-5
