"""The 1 Mb pooling maps of init_params (csrc/pool.cu) against torch's avg_pool2d on the same
tiles (parafac2_intergrative.py:102-151: stride ll, no padding, the floor of each side), and
the unpooling as its exact transpose."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib

pytestmark = pytest.mark.gpu
CUDA = torch.device("cuda")


@pytest.mark.parametrize("ll", [2, 3])
def test_pool_rows_is_avg_pool2d_and_unpool_its_transpose(ll):
    from fh_gb300.sparse_for_schic import tile_table
    rng = np.random.default_rng(ll)
    # tiles of uneven shapes (rows, width) laid out one after another in band rows
    shapes = [(25, 37), (25, 41), (24, 33), (7, 12), (1, 5)]
    recs, xoff = [], 0
    for b, n in shapes:
        recs.append((0, 0, b, n, 0, 0, 1, 0, xoff, 0, 0))
        xoff += b * n
    tiles = np.array(recs, dtype=_lib.TILE_DTYPE)
    tdev = torch.from_numpy(tiles.view(np.uint8).copy()).to(CUDA)
    pr = [0]
    for b, n in shapes:
        pr.append(pr[-1] + (b // ll) * (n // ll))
    prow0 = torch.tensor(pr, dtype=torch.int64, device=CUDA)
    lls = torch.full((len(shapes),), ll, dtype=torch.int32, device=CUDA)
    m, x0 = 5, 0
    W = torch.from_numpy(rng.standard_normal((xoff, m)).astype(np.float32)).to(CUDA)
    out = torch.empty((pr[-1], m), dtype=torch.float32, device=CUDA)
    P = _lib.ptr
    _lib.call("fh_pool_rows", P(tdev), len(shapes), P(prow0), P(lls), x0, P(W), m, m, P(out), m,
              _lib.stream_ptr())
    ref = []
    for (b, n), (*_, xo, _b, _u) in zip(shapes, recs):
        if b < ll or n < ll:               # no whole block: no pooled rows (torch refuses)
            continue
        blk = W[xo:xo + b * n].view(b, n, m).permute(2, 0, 1)[:, None]     # m x 1 x b x n
        pooled = torch.nn.functional.avg_pool2d(blk, ll, ll, padding=0, ceil_mode=False)
        ref.append(pooled[:, 0].reshape(m, -1).T)
    ref = torch.cat(ref, dim=0)
    torch.cuda.synchronize()
    assert torch.allclose(out, ref, rtol=1e-6, atol=1e-6)
    # unpool is the transpose: <pool(W), Q> = <W, unpool(Q)>
    Q = torch.from_numpy(rng.standard_normal((pr[-1], m)).astype(np.float32)).to(CUDA)
    back = torch.empty((xoff, m), dtype=torch.float32, device=CUDA)
    _lib.call("fh_unpool_rows", P(tdev), len(shapes), P(prow0), P(lls), x0, xoff, P(Q), m, m,
              P(back), m, _lib.stream_ptr())
    torch.cuda.synchronize()
    lhs = float((out.double() * Q.double()).sum())
    rhs = float((W.double() * back.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + 1)
