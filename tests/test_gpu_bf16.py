"""GPU checks of the bf16 tensor-core form of the X passes (tcgen05 + TMA kernels).

Tolerances (relative Frobenius error):
  split hi|lo            |x - (hi + lo)| <= 2^-16 |x| per element
  fh_xe_bf16, fh_xg_bf16 1e-5 against an fp64 product of the same bf16 X and the exact fp32
                         small operand (the split carries it to 2^-16, the fp32 accumulator
                         adds ~1e-7 sqrt(K))
  fh_rwr_tiles_bf16      plane 0 bit-identical to bf16(fh_rwr_tiles_f32), plane 1 to the bf16
                         of the residual
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib
import golden_io as G
from gpu_util import datasets_from

pytestmark = pytest.mark.gpu

CUDA = torch.device("cuda")
P = _lib.ptr


def sp():
    return _lib.stream_ptr()


def rel64(a, b):
    a = a.double()
    b = b.double()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def split(x):
    n, rp = x.shape
    out = torch.empty((n, 2 * rp), dtype=torch.bfloat16, device=CUDA)
    _lib.call("fh_split_bf16", P(x), n, rp, rp, P(out), sp())
    return out


def make_x16(ct, rows, seed, planes=1):
    """X as bf16 planes [planes][ct][ldx] and its exact value (the sum of the planes)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    ldx = int(math.ceil(rows / 128) * 128)
    X = torch.zeros((ct, ldx), dtype=torch.float32)
    X[:, :rows] = torch.rand((ct, rows), generator=g) * torch.rand((ct, 1), generator=g)
    hi = X.to(torch.bfloat16)
    pl = [hi]
    if planes == 2:
        pl.append((X - hi.float()).to(torch.bfloat16))
    X16 = torch.stack(pl).contiguous().to(CUDA)
    return X16, ldx, X16.double().sum(0)


def test_split_bf16_exact_to_16_bits():
    x = torch.randn((333, 64), device=CUDA) * torch.logspace(-3, 3, 64, device=CUDA)
    s = split(x)
    hi, lo = s[:, :64].float(), s[:, 64:].float()
    err = (x - (hi + lo)).abs() / x.abs().clamp_min(1e-30)
    assert float(err.max()) <= 2.0 ** -16


@pytest.mark.parametrize("planes", [1, 2])
@pytest.mark.parametrize("rp,ct,c,rows", [(64, 300, 260, 1000), (64, 2000, 2000, 40000),
                                          (32, 190, 130, 777), (128, 400, 333, 3001)])
def test_xe_bf16(rp, ct, c, rows, planes):
    X16, ldx, Xv = make_x16(ct, rows, 1 + rp, planes)
    E = torch.randn((c, rp), device=CUDA)
    E2 = split(E)
    W = torch.full((rows, rp), float("nan"), device=CUDA)
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    _lib.call("fh_xe_bf16", P(X16), ldx, ct, planes, c, rows, P(E2), rp, 0, P(W), P(st), sp())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = Xv[:c, :rows].T @ E.double()
    assert rel64(W, ref) < 1e-5


@pytest.mark.parametrize("planes", [1, 2])
@pytest.mark.parametrize("rp,ct,n,rows", [(64, 300, 300, 1000), (64, 2000, 1900, 40000),
                                          (32, 190, 130, 20000), (128, 400, 400, 3001)])
def test_xg_bf16(rp, ct, n, rows, planes):
    X16, ldx, Xv = make_x16(ct, rows, 7 + rp, planes)
    Gt = torch.randn((rows, rp), device=CUDA)
    G2 = split(Gt)
    splits = _lib.value("fh_xg_bf16_splits", n, rows)
    assert splits >= 1
    partial = torch.empty((splits, n, rp), device=CUDA)
    out = torch.full((n, rp), float("nan"), device=CUDA)
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    _lib.call("fh_xg_bf16", P(X16), ldx, ct, planes, n, rows, P(G2), rp, splits, 0, P(partial),
              P(out), 0, P(st), sp())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = Xv[:n, :rows] @ Gt.double()
    assert rel64(out, ref) < 1e-5


def test_xpass_bf16_deterministic():
    X16, ldx, _ = make_x16(1000, 30000, 3, 2)
    Gt = torch.randn((30000, 64), device=CUDA)
    G2 = split(Gt)
    splits = _lib.value("fh_xg_bf16_splits", 1000, 30000)
    partial = torch.empty((splits, 1000, 64), device=CUDA)
    outs = []
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    for _ in range(2):
        out = torch.empty((1000, 64), device=CUDA)
        _lib.call("fh_xg_bf16", P(X16), ldx, 1000, 2, 1000, 30000, P(G2), 64, splits, 0,
                  P(partial), P(out), 0, P(st), sp())
        outs.append(out)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1])


def test_rwr_tiles_bf16_planes_are_split_fp32():
    from fh_gb300.engine import FitEngine
    z = G.load("rwr_tiles.npz")
    ds = datasets_from(z, resolution=1000000)
    eng = FitEngine(ds, 4, {d.chrom: 2 for d in ds}, [3] * len(ds), CUDA)
    X16 = torch.zeros((2, eng.Ct, eng.ldx), dtype=torch.bfloat16, device=CUDA)
    ss = torch.zeros_like(eng.sumsq)
    _lib.call("fh_rwr_tiles_bf16", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
              eng.max_width, P(eng.store.entries), P(eng.store.offsets), P(X16), eng.ldx,
              eng.Ct * eng.ldx, P(ss), P(eng.status), sp())
    torch.cuda.synchronize()
    hi = eng.X.to(torch.bfloat16)
    assert torch.equal(X16[0], hi)
    assert torch.equal(X16[1], (eng.X - hi.float()).to(torch.bfloat16))
    np.testing.assert_allclose(ss.cpu().numpy(), eng.sumsq.cpu().numpy(), rtol=1e-4)


@pytest.mark.parametrize("planes,form", [(1, 1), (2, 1), (1, 2), (2, 2)])
def test_rwr_tiles_tc_matches_fp32(planes, form):
    """tcgen05 RWR (split bf16 products) against the fp32 CUDA-core RWR on the golden tiles."""
    from fh_gb300.engine import FitEngine
    z = G.load("rwr_tiles.npz")
    ds = datasets_from(z, resolution=1000000)
    eng = FitEngine(ds, 4, {d.chrom: 2 for d in ds}, [3] * len(ds), CUDA)
    X16 = torch.zeros((planes, eng.Ct, eng.ldx), dtype=torch.bfloat16, device=CUDA)
    ss = torch.zeros_like(eng.sumsq)
    _lib.call("fh_rwr_tiles_tc", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
              eng.max_width, P(eng.store.entries), P(eng.store.offsets), P(X16), eng.ldx,
              eng.Ct * eng.ldx if planes == 2 else 0, P(ss), form, P(eng.status), sp())
    torch.cuda.synchronize()
    assert int(eng.status.item()) == 0
    got = X16.double().sum(0)
    tol = 1e-4 if planes == 2 else 4e-3
    assert rel64(got, eng.X.double()) < tol
    np.testing.assert_allclose(ss.cpu().numpy(), eng.sumsq.cpu().numpy(), rtol=10 * tol)


@pytest.mark.parametrize("epochs,band,form", [(0, 20, 1), (1, 20, 1), (6, 20, 1), (0, 20, 2),
                                              (1, 20, 2), (6, 20, 2), (0, 70, 1), (6, 70, 1)])
def test_rwr_tiles_tc_full_tiles(epochs, band, form):
    """125-row bin batches of a 1 Mb genome-like chromosome, 300 cells: band 20 (widths up to
    145, padded to 192) in both forms, band 70 (widths up to 195, padded to 256) in the form
    with P in shared memory; the pipelined form refuses it."""
    from fh_gb300 import synth
    from fh_gb300.engine import FitEngine
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    w = synth.workload("c2")
    w.n_cells = 300
    w.band = band
    w.chrom_bins = w.chrom_bins[:2]
    w.chrom_names = w.chrom_names[:2]
    coo, _ = synth.generate(w, seed=3)
    ds = [Chrom_Dataset(Sparse(i, v, s, copy=False), *synth.recommend_batches(w, nb, w.n_cells),
                        compact=True, flank=w.band, chrom=nm, resolution=w.resolution)
          for (i, v, s), nm, nb in zip(coo, w.chrom_names, w.chrom_bins)]
    eng = FitEngine(ds, 64, {d.chrom: 64 for d in ds}, [epochs] * len(ds), CUDA)
    X16 = torch.zeros((2, eng.Ct, eng.ldx), dtype=torch.bfloat16, device=CUDA)
    ss = torch.zeros_like(eng.sumsq)
    args = (P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows, eng.max_width,
            P(eng.store.entries), P(eng.store.offsets), P(X16), eng.ldx, eng.Ct * eng.ldx,
            P(ss))
    _lib.call("fh_rwr_tiles_tc", *args, form, P(eng.status), sp())
    torch.cuda.synchronize()
    assert int(eng.status.item()) == 0
    assert rel64(X16.double().sum(0), eng.X.double()) < 1e-4
    assert float(X16[:, :, eng.rows:].abs().max()) == 0.0
    if band == 70:
        assert eng.max_width > 192
        assert _lib.value("fh_rwr_tiles_tc", *args, 2, P(eng.status), sp()) == 2  # unsupported
