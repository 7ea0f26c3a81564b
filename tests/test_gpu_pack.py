"""GPU input packing (csrc/pack.cu, fh_gb300.pack) against the reference's own packing and the
oracle's restatement of it.

Indices and shapes must be bit-exact (integer work).  Values within 1e-6 relative per entry:
the kernels sum each cell's coverage and the clip's moments in fp64 where the reference sums
fp32 in numpy's order, so a value may differ by an ulp or two (measured: see the prints).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import fh_oracle as O
import golden_io as G

pytestmark = pytest.mark.gpu


def _check(got, want):
    idx, val, shape = got
    ridx, rval, rshape = want
    assert tuple(shape) == tuple(rshape)
    np.testing.assert_array_equal(idx.cpu().numpy(), np.asarray(ridx))
    v = val.cpu().numpy().astype(np.float64)
    r = np.asarray(rval, dtype=np.float64)
    rel = np.abs(v - r) / np.maximum(np.abs(r), 1e-30)
    print("packed entries %d, max relative difference %.2e, equal %.4f" %
          (len(r), rel.max() if len(r) else 0.0, float(np.mean(v == r)) if len(r) else 1.0))
    assert len(r) == 0 or rel.max() < 1e-6


@pytest.mark.parametrize("k,case", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_pack_matches_reference_fixture(k, case):
    from fh_gb300.pack import pack_chromosome
    z = G.load("pack.npz")
    n = int(z["n_cells"])
    cells = [(z["raw%d_cell%d" % (k, c)][0], z["raw%d_cell%d" % (k, c)][1],
              z["raw%d_val%d" % (k, c)]) for c in range(n)]
    merge, off_diag = (int(v) for v in z["out%d_%d_args" % (k, case)])
    ref = "out%d_%d" % (k, case)
    got = pack_chromosome(cells, int(z["raw%d_nbin" % k]), z["reorder"], off_diag, merge)
    _check(got, (z[ref + "_idx"], z[ref + "_val"], z[ref + "_shape"]))


def _random_cells(rng, n_cells, nbin, band, empty=(), dead_bins=()):
    cells = []
    for c in range(n_cells):
        if c in empty:
            cells.append((np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32)))
            continue
        m = int(rng.integers(50, 400))
        r = rng.integers(0, nbin, m)
        d = rng.integers(-band, band + 1, m)
        cc = np.clip(r + d, 0, nbin - 1)
        keep = ~np.isin(r, dead_bins) & ~np.isin(cc, dead_bins)
        r, cc = r[keep], cc[keep]
        rr, ccc = np.concatenate([r, cc]), np.concatenate([cc, r])       # symmetric
        key = rr * nbin + ccc
        u, inv = np.unique(key, return_inverse=True)
        v = np.bincount(inv).astype(np.float32)                           # counts
        cells.append(((u // nbin).astype(np.int32), (u % nbin).astype(np.int32), v))
    return cells


@pytest.mark.parametrize("merge,off_diag", [(1, 10), (3, 4), (2, 0)])
def test_pack_matches_oracle_on_ragged_cells(merge, off_diag):
    """300 cells of ragged size over 257 bins, two empty cells, dead bins, a shuffled order."""
    from fh_gb300.pack import pack_chromosome
    rng = np.random.default_rng(merge * 10 + off_diag)
    cells = _random_cells(rng, 300, 257, 25, empty=(3, 77), dead_bins=(0, 1, 100, 101, 256))
    order = rng.permutation(300)
    want = O.pack_chromosome(cells, 257, order, off_diag, merge)
    _check(pack_chromosome(cells, 257, order, off_diag, merge), want)


def test_pack_rejects_bad_coordinates():
    from fh_gb300 import _lib
    from fh_gb300.pack import pack_chromosome
    cells = [(np.array([0, 5], np.int32), np.array([0, 40], np.int32), np.ones(2, np.float32))]
    with pytest.raises(_lib.FHError):
        pack_chromosome(cells, 20, [0], 3)          # column 40 past 20 bins
    with pytest.raises(_lib.FHError):
        pack_chromosome(cells, 50, [1], 3)          # no raw cell 1
