"""Accuracy of the long sums in the X passes, against fp64 products of the same operands.

At 10,000 cells x 500 kb each entry of W = X^T E sums 10,000 cells and each split of
S^T = X G^T sums ~35,000 band rows.  The fitted embedding inherits the rounding of these sums
(the meta polar multiplies the error of S^T by its condition number), so the passes sum in
short runs folded into Kahan-compensated running sums.  These checks run both forms at those
K lengths on RWR-like data (non-negative, heavy-tailed, cell-scaled X; E with orthonormal
columns, so every column but the first cancels heavily) and state each error against an fp64
product of exactly the operands the kernel read:

  fp32 form      X and the small operand in fp32; the FMA products are exact, so the error is
                 the summation's alone
  bf16x2 form    X as two bf16 planes (the fp64 reference uses their exact sum) and the small
                 operand split hi | lo to 16 significant bits inside the pass; "split floor" is
                 the error that split alone causes (fp64 product with the split operand), the
                 least any summation order can reach

Measured errors print as one JSON line (and go to $FH_PRECISION_OUT/accumulation.json when
that names a folder).
"""
import json
import math
import os

import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib

pytestmark = pytest.mark.gpu

CUDA = torch.device("cuda")
P = _lib.ptr
RESULTS = {}


def sp():
    return _lib.stream_ptr()


def rel(a, b):
    a, b = a.double(), b.double()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def rwr_like(ct, rows, seed):
    """[ct][ldx] fp32, non-negative and heavy-tailed per cell (log-normal cell scales), zero
    padding past rows."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    ldx = int(math.ceil(rows / 128) * 128)
    X = torch.zeros((ct, ldx), dtype=torch.float32)
    scale = torch.exp(0.8 * torch.randn((ct, 1), generator=g))
    X[:, :rows] = torch.rand((ct, rows), generator=g) ** 3 * scale
    return X.to(CUDA), ldx


def planes_of(X):
    hi = X.to(torch.bfloat16)
    lo = (X - hi.float()).to(torch.bfloat16)
    return torch.stack([hi, lo]).contiguous(), hi.double() + lo.double()


def split(x):
    n, rp = x.shape
    out = torch.empty((n, 2 * rp), dtype=torch.bfloat16, device=CUDA)
    _lib.call("fh_split_bf16", P(x), n, rp, rp, P(out), sp())
    return out


def unsplit(x2, rp):
    return x2[:, :rp].double() + x2[:, rp:].double()


def record(name, errs):
    RESULTS[name] = errs
    print(json.dumps({name: errs}))
    d = os.environ.get("FH_PRECISION_OUT", "")
    if d and os.path.isdir(d):
        with open(os.path.join(d, "accumulation.json"), "w") as f:
            json.dump(RESULTS, f, indent=1)


def test_xe_long_sum_10000_cells():
    """W = X^T E over 10,000 cells (one K range of 157 chunks)."""
    C, rows, rp = 10000, 2048, 64
    X, ldx = rwr_like(C, rows, 3)
    E, _ = torch.linalg.qr(torch.randn((C, rp), dtype=torch.float64, device=CUDA))
    E = E.float().contiguous()
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    errs = {}
    W = torch.empty((rows, rp), device=CUDA)
    _lib.call("fh_xe_f32", P(X), ldx, C, rows, P(E), rp, P(W), sp())
    errs["fp32"] = rel(W, X[:, :rows].double().T @ E.double())
    X16, Xv = planes_of(X)
    E2 = split(E)
    ref = Xv[:, :rows].T @ E.double()
    errs["bf16x2_split_floor"] = rel(Xv[:, :rows].T @ unsplit(E2, rp), ref)
    for fold in (1, 8, 1 << 20):
        _lib.call("fh_xe_bf16", P(X16), ldx, C, 2, C, rows, P(E2), rp, fold, P(W), P(st), sp())
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        errs["bf16x2_fold%d" % fold] = rel(W, ref)
    record("xe_10000_cells", errs)
    assert errs["fp32"] < 2e-7
    # folded runs stay within 2x of the split's own error; one run per item is the old form
    assert errs["bf16x2_fold8"] < 2 * errs["bf16x2_split_floor"] + 1e-7
    assert errs["bf16x2_fold1"] < 2 * errs["bf16x2_split_floor"] + 1e-7


def test_xg_long_sum_35000_rows_per_split():
    """S^T = X G^T with 4 splits of 35,840 band rows (560 chunks each), as at 10,000 cells."""
    n, rows, rp, splits = 256, 4 * 35840, 64, 4
    X, ldx = rwr_like(n, rows, 5)
    Gt = (torch.randn((rows, rp), device=CUDA) / math.sqrt(rows)).contiguous()
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    partial = torch.empty((splits, n, rp), device=CUDA)
    out = torch.empty((n, rp), device=CUDA)
    errs = {}
    _lib.call("fh_xg_f32", P(X), ldx, n, rows, P(Gt), rp, splits, P(partial), P(out), 0, sp())
    errs["fp32"] = rel(out, X[:, :rows].double() @ Gt.double())
    X16, Xv = planes_of(X)
    G2 = split(Gt)
    ref = Xv[:, :rows] @ Gt.double()
    errs["bf16x2_split_floor"] = rel(Xv[:, :rows] @ unsplit(G2, rp), ref)
    for fold in (1, 8, 1 << 20):
        _lib.call("fh_xg_bf16", P(X16), ldx, n, 2, n, rows, P(G2), rp, splits, fold,
                  P(partial), P(out), 0, P(st), sp())
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        errs["bf16x2_fold%d" % fold] = rel(out, ref)
    record("xg_35840_rows_per_split", errs)
    assert errs["fp32"] < 2e-7
    assert errs["bf16x2_fold8"] < 2 * errs["bf16x2_split_floor"] + 1e-7
    assert errs["bf16x2_fold1"] < 2 * errs["bf16x2_split_floor"] + 1e-7


@pytest.mark.parametrize("rp", [32, 128])
def test_fold_every_rank(rp):
    """Folded runs at the other ranks (rank 128 has eight epilogue warps, two column groups
    per TMEM lane quarter); fold = 3 leaves a short last run in every item."""
    C, rows = 3000, 1000
    X, ldx = rwr_like(C, rows, 11 + rp)
    E = torch.randn((C, rp), device=CUDA) / math.sqrt(C)
    X16, Xv = planes_of(X)
    E2 = split(E)
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    W = torch.full((rows, rp), float("nan"), device=CUDA)
    _lib.call("fh_xe_bf16", P(X16), ldx, C, 2, C, rows, P(E2), rp, 3, P(W), P(st), sp())
    Gt = torch.randn((rows, rp), device=CUDA) / math.sqrt(rows)
    G2 = split(Gt)
    splits = _lib.value("fh_xg_bf16_splits", C, rows)
    partial = torch.empty((splits, C, rp), device=CUDA)
    out = torch.full((C, rp), float("nan"), device=CUDA)
    _lib.call("fh_xg_bf16", P(X16), ldx, C, 2, C, rows, P(G2), rp, splits, 3, P(partial),
              P(out), 0, P(st), sp())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    e_w = rel(W, Xv[:, :rows].T @ unsplit(E2, rp))
    e_s = rel(out, Xv[:, :rows] @ unsplit(G2, rp))
    record("fold3_rank%d" % rp, {"xe_vs_split_operands": e_w, "xg_vs_split_operands": e_s})
    assert e_w < 1e-6 and e_s < 1e-6
