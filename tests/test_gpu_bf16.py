"""GPU checks of the bf16 tensor-core form of the X passes (tcgen05 + TMA kernels).

Tolerances (relative Frobenius error):
  split hi|lo            |x - (hi + lo)| <= 2^-16 |x| per element
  fh_xe_bf16, fh_xg_bf16 1e-5 against an fp64 product of the same bf16 X and the exact fp32
                         small operand (the split carries it to 2^-16, the fp32 accumulator
                         adds ~1e-7 sqrt(K))
  fh_rwr_tiles_bf16      bit-identical to bf16(fh_rwr_tiles_f32)
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


def make_x16(ct, rows, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    ldx = int(math.ceil(rows / 128) * 128)
    X = torch.zeros((ct, ldx), dtype=torch.float32)
    X[:, :rows] = torch.rand((ct, rows), generator=g) * torch.rand((ct, 1), generator=g)
    return X.to(torch.bfloat16).to(CUDA), ldx


def test_split_bf16_exact_to_16_bits():
    x = torch.randn((333, 64), device=CUDA) * torch.logspace(-3, 3, 64, device=CUDA)
    s = split(x)
    hi, lo = s[:, :64].float(), s[:, 64:].float()
    err = (x - (hi + lo)).abs() / x.abs().clamp_min(1e-30)
    assert float(err.max()) <= 2.0 ** -16


@pytest.mark.parametrize("rp,ct,c,rows", [(64, 300, 260, 1000), (64, 2000, 2000, 40000),
                                          (32, 190, 130, 777), (128, 400, 333, 3001)])
def test_xe_bf16(rp, ct, c, rows):
    X16, ldx = make_x16(ct, rows, 1 + rp)
    E = torch.randn((c, rp), device=CUDA)
    E2 = split(E)
    W = torch.full((rows, rp), float("nan"), device=CUDA)
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    _lib.call("fh_xe_bf16", P(X16), ldx, ct, c, rows, P(E2), rp, P(W), P(st), sp())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = X16[:c, :rows].double().T @ E.double()
    assert rel64(W, ref) < 1e-5


@pytest.mark.parametrize("rp,ct,n,rows", [(64, 300, 300, 1000), (64, 2000, 1900, 40000),
                                          (32, 190, 130, 20000), (128, 400, 400, 3001)])
def test_xg_bf16(rp, ct, n, rows):
    X16, ldx = make_x16(ct, rows, 7 + rp)
    Gt = torch.randn((rows, rp), device=CUDA)
    G2 = split(Gt)
    splits = _lib.value("fh_xg_bf16_splits", n, rows)
    assert splits >= 1
    partial = torch.empty((splits, n, rp), device=CUDA)
    out = torch.full((n, rp), float("nan"), device=CUDA)
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    _lib.call("fh_xg_bf16", P(X16), ldx, ct, n, rows, P(G2), rp, splits, P(partial), P(out),
              P(st), sp())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = X16[:n, :rows].double() @ Gt.double()
    assert rel64(out, ref) < 1e-5


def test_xpass_bf16_deterministic():
    X16, ldx = make_x16(1000, 30000, 3)
    Gt = torch.randn((30000, 64), device=CUDA)
    G2 = split(Gt)
    splits = _lib.value("fh_xg_bf16_splits", 1000, 30000)
    partial = torch.empty((splits, 1000, 64), device=CUDA)
    outs = []
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    for _ in range(2):
        out = torch.empty((1000, 64), device=CUDA)
        _lib.call("fh_xg_bf16", P(X16), ldx, 1000, 1000, 30000, P(G2), 64, splits, P(partial),
                  P(out), P(st), sp())
        outs.append(out)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1])


def test_rwr_tiles_bf16_is_rounded_fp32():
    from fh_gb300.engine import FitEngine
    z = G.load("rwr_tiles.npz")
    ds = datasets_from(z, resolution=1000000)
    eng = FitEngine(ds, 4, {d.chrom: 2 for d in ds}, [3] * len(ds), CUDA)
    X16 = torch.zeros((eng.Ct, eng.ldx), dtype=torch.bfloat16, device=CUDA)
    ss = torch.zeros_like(eng.sumsq)
    _lib.call("fh_rwr_tiles_bf16", P(eng.tiles_dev), eng.n_tiles, eng.Ct, eng.max_rows,
              eng.max_width, P(eng.store.entries), P(eng.store.offsets), P(X16), eng.ldx, P(ss),
              P(eng.status), sp())
    torch.cuda.synchronize()
    assert torch.equal(X16, eng.X.to(torch.bfloat16))
    np.testing.assert_allclose(ss.cpu().numpy(), eng.sumsq.cpu().numpy(), rtol=1e-2)
