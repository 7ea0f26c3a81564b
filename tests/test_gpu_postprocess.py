"""GPU embedding post-processing (csrc/embed.cu, fh_gb300.postprocess) against the reference's
fetch_cell_embedding / correct_batch_linear outputs and the oracle's restatement.

Tolerances: the quantile transform is fp64 integer-order work with the reference's operation
order, so it must be bit-exact.  The embedding product is fp32 as the reference's (1e-6).
The truncated SVDs are exact in fp64 here and randomized fp32 in the reference: against the
oracle's exact fp64 SVD 1e-5, against the reference within its own sketch error (5e-5), with
the reference's component signs (no sign alignment).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import fh_oracle as O
import golden_io as G

pytestmark = pytest.mark.gpu

KEYS = ["embed_all", "embed_raw", "embed_l2_norm", "embed_correct_coverage_fh",
        "embed_l2_norm_correct_coverage_fh", "embed_correct_batch",
        "embed_l2_norm_correct_batch"]


def _case(z, k):
    E = z["c%d_E" % k]
    Ds = [z["c%d_D%d" % (k, i)] for i in range(int(z["c%d_nD" % k]))]
    return E, Ds, z["c%d_readcount" % k], int(z["c%d_final_dim" % k]), z["c%d_reorder" % k]


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("restore", [False, True])
def test_fetch_cell_embedding_matches_reference_and_oracle(k, restore):
    from fh_gb300.postprocess import EmbeddingPostprocess
    z = G.load("postprocess.npz")
    E, Ds, rc, fd, reorder = _case(z, k)
    pp = EmbeddingPostprocess(E, Ds, rc.reshape(-1, 1), {"batch": z["c%d_batch" % k]},
                              reorder, rank=fd)
    st = pp.fetch_cell_embedding(final_dim=fd, restore_order=restore)
    pp.correct_batch_linear("batch", True)
    want = O.fetch_cell_embedding(E, Ds, rc, fd, restore, reorder)
    O.correct_batch_linear(want, z["c%d_batch" % k], "batch", True, reorder)
    key = "c%d_r%d_" % (k, int(restore))
    np.testing.assert_array_equal(pp.label_info["coverage_fh"], z[key + "coverage_fh"])
    errs = {}
    for name in KEYS:
        e_ref = O.rel_err(st[name], z[key + name])
        e_orc = O.rel_err(st[name], want[name])
        errs[name] = (e_ref, e_orc)
        tol = 1e-6 if name == "embed_all" else 1e-5
        assert e_orc < tol, (name, e_orc)
        assert e_ref < 5e-5, (name, e_ref)
    print({n: "%.1e / %.1e" % v for n, v in errs.items()})


@pytest.mark.parametrize("n,nq", [(1, 100), (2, 100), (97, 100), (1000, 100), (20000, 100),
                                  (5000, 7)])
def test_quantile_uniform_bit_exact(n, nq):
    from fh_gb300.postprocess import quantile_transform_uniform
    rng = np.random.default_rng(n + nq)
    x = np.round(np.exp(rng.normal(9, 1.2, n)) / 40) * 40          # many ties
    got = quantile_transform_uniform(x, nq).cpu().numpy()
    np.testing.assert_array_equal(got, O.quantile_uniform(x, nq))


@pytest.mark.parametrize("kind", ["float", "labels"])
@pytest.mark.parametrize("back", [False, True])
def test_linear_residual_matches_oracle(kind, back):
    from fh_gb300.postprocess import linear_residual
    rng = np.random.default_rng(3)
    C, m = 700, 90
    Y = rng.standard_normal((C, m)).astype(np.float32) + 2.0
    if kind == "float":
        V = np.stack([rng.uniform(0, 1, C), rng.standard_normal(C)], axis=1)
    else:   # one-hot columns that sum to the intercept: the minimum-norm coefficients
        V = O.one_hot(np.array(["a", "b", "c", "d"])[rng.integers(0, 4, C)])
    got = linear_residual(V, Y, back).cpu().numpy()
    assert O.rel_err(got, O.linear_residual(V, Y, back)) < 1e-6


def test_range_svd_with_dependent_columns_and_zero_rows():
    """A span given with a repeated column and a column of zeros (dropped directions), and
    rows of zeros in the embedding (unchanged by the normalisation)."""
    from fh_gb300.postprocess import truncated_svd_in_span, l2_normalize
    rng = np.random.default_rng(8)
    C, R, m, k = 500, 10, 60, 7
    E = rng.standard_normal((C, R)).astype(np.float32) * np.linspace(4, 1, R)[None]
    E[:5] = 0
    M = rng.standard_normal((R, m)).astype(np.float32)
    Y = E @ M
    F = np.concatenate([E, E[:, :2], np.zeros((C, 1), np.float32)], axis=1)
    got, sig = truncated_svd_in_span(F, Y, k)
    want = O.truncated_svd(Y, k)
    assert O.rel_err(got.cpu().numpy(), want) < 1e-5
    s_ref = np.linalg.svd(Y.astype(np.float64), compute_uv=False)[:k]
    assert O.rel_err(sig.cpu().numpy(), s_ref) < 1e-9
    l2 = l2_normalize(got).cpu().numpy()
    assert np.all(got.cpu().numpy()[:5] == 0) and np.all(l2[:5] == 0)
    want[:5] = 0      # the fp64 SVD leaves ~1e-17 in the zero rows, which normalising would blow up
    assert O.rel_err(l2, O.l2_rows(want)) < 1e-5


def test_bad_input_fails_loudly():
    from fh_gb300 import _lib
    from fh_gb300.postprocess import truncated_svd_in_span
    Y = np.ones((10, 4), np.float32)
    with pytest.raises(_lib.FHError):
        truncated_svd_in_span(np.ones((10, 2), np.float32), Y, 3)     # k above the span's width
    with pytest.raises(_lib.FHError):
        truncated_svd_in_span(np.ones((10, 2), np.float32), Y, 2, device="cpu")
