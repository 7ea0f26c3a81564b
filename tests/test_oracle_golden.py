"""Pins the oracle (CPU restatement) against the reference's own outputs (tests/golden)."""
import numpy as np
import pytest

from oracle import fh_oracle as O
import golden_io as G


def test_tile_layout_and_densify_match_reference_fetch():
    z = G.load("rwr_tiles.npz")
    datas = G.chrom_datas(z, O)
    for k in range(int(z["n_tiles"])):
        ci, bi, cj, s0, s1, _ = z["t%d_meta" % k]
        d = datas[ci]
        bb = d.layout()[bi]
        assert (bb.local.start, bb.local.stop) == (s0, s1)
        x = d.tile(bb, d.cells()[cj], np.float32)
        np.testing.assert_array_equal(x, z["t%d_x" % k])


@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 1e-5)])
def test_partial_rwr_matches_reference(dtype, tol):
    z = G.load("rwr_tiles.npz")
    for k in range(int(z["n_tiles"])):
        _, _, _, s0, s1, n_auto = z["t%d_meta" % k]
        x = z["t%d_x" % k].astype(dtype)
        y3, _ = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=3)
        assert O.rel_err(y3, z["t%d_y3" % k]) < tol
        ya, na = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=-1, final_transpose=False,
                               return_rwr_iter=True)
        assert na == n_auto
        assert O.rel_err(ya, z["t%d_yauto" % k]) < tol


@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 1e-5)])
def test_partial_rwr_with_conv_matches_reference(dtype, tol):
    """do_conv=True: the 3 x 3 mean (partial_rwr.py:79-83) before the walk, and alone."""
    z = G.load("rwr_conv_tiles.npz")
    for k in range(int(z["n_tiles"])):
        _, _, _, s0, s1, n_auto = z["t%d_meta" % k]
        x = z["t%d_x" % k].astype(dtype)
        y3, _ = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=3, do_conv=True)
        assert O.rel_err(y3, z["t%d_y3" % k]) < tol
        ya, na = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=-1, final_transpose=False,
                               return_rwr_iter=True, do_conv=True)
        assert na == n_auto
        assert O.rel_err(ya, z["t%d_yauto" % k]) < tol
        y0, _ = O.partial_rwr(x.copy(), s0, s1, do_rwr=False, do_conv=True)
        assert O.rel_err(y0, z["t%d_y0" % k]) < tol


@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 1e-5)])
def test_partial_rwr_with_col_matches_reference(dtype, tol):
    """do_col=True (partial_rwr.py:131-138): the symmetrised, row-normalised Q applied to the
    tile divided by the coverage argument (inf entries zero their columns)."""
    z = G.load("rwr_col_tiles.npz")
    for k in range(int(z["n_tiles"])):
        _, _, _, s0, s1, n_auto = z["t%d_meta" % k]
        x = z["t%d_x" % k].astype(dtype)
        cov = z["t%d_cov" % k].astype(dtype)
        y3, _ = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=3, do_col=True, bin_cov=cov)
        assert O.rel_err(y3, z["t%d_y3" % k]) < tol
        ya, na = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=-1, final_transpose=False,
                               return_rwr_iter=True, do_col=True, bin_cov=cov)
        assert na == n_auto
        assert O.rel_err(ya, z["t%d_yauto" % k]) < tol
        yc, _ = O.partial_rwr(x.copy(), s0, s1, force_rwr_epochs=3, do_col=True, bin_cov=cov,
                              do_conv=True)
        assert O.rel_err(yc, z["t%d_yconv3" % k]) < tol


def test_col_coverage_matches_reference_init():
    """bin_cov of init_params (parafac2_intergrative.py:96-142, 266-267) on the small workload."""
    z = G.load("als_col_small.npz")
    datas = G.chrom_datas(z, O)
    cov = O.col_coverage(datas, np.float32)
    for k, c in enumerate(cov):
        ref = z["init_bincov%d" % k]
        np.testing.assert_array_equal(np.isinf(c), np.isinf(ref))
        fin = np.isfinite(ref)
        assert O.rel_err(c[fin], ref[fin]) < 2e-6


@pytest.mark.parametrize("n", [1, 3])
def test_parafac_matches_reference(n):
    z = G.load("parafac.npz")
    f, ln, lx = O.parafac(z["X"], 6, n_iter_max=n, init=[z["A0"], z["B0"], z["D0"]])
    for a, name in zip(f, "ABD"):
        assert O.rel_err(a, z["%s%d" % (name, n)]) < 1e-4
    assert abs(ln - float(z["ln%d" % n])) / abs(float(z["ln%d" % n])) < 1e-5
    assert abs(lx - float(z["lx%d" % n])) / abs(float(z["lx%d" % n])) < 1e-5


def _oracle_from(z, prefix="init", dtype=np.float64, do_conv=False, do_col=False):
    datas = G.chrom_datas(z, O)
    A, B, D, E, n_i = G.state(z, prefix, len(datas))
    cov = [z["init_bincov%d" % k] for k in range(len(datas))] if do_col else None
    bad = [z["init_badbincov%d" % k] if "init_badbincov%d" % k in z else None
           for k in range(len(datas))] if do_col else None
    do_rwr = bool(int(z["do_rwr"])) if "do_rwr" in z else True
    return O.ALSOracle(datas, int(z["rank"]), A, B, D, E, n_i, dtype=dtype, do_conv=do_conv,
                       do_col=do_col, bin_cov_list=cov, bad_bin_cov_list=bad, do_rwr=do_rwr)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_one_update_matches_reference(dtype):
    """One update_meta_embedding_interactions call from the reference's init state.
    Well-conditioned outputs agree to 1e-5; the polar factors U agree to the reference's
    own fp32 SVD error, which grows with the conditioning of the per-bin matrices."""
    z = G.load("als_small.npz")
    orc = _oracle_from(z, dtype=dtype)
    U, Y, exU, exV, tn = orc.update(first_iter=True)
    assert O.rel_err(tn, z["it1_tnorm"]) < 1e-5
    assert O.rel_err(exU, z["it1_exU"]) < 1e-5
    assert abs(exV - float(z["it1_exV"])) / abs(float(z["it1_exV"])) < 1e-5
    errs = [O.rel_err(U[ci][bi], z["it1_U%d_%d" % (ci, bi)])
            for ci in range(len(U)) for bi in range(len(U[ci]))]
    assert np.median(errs) < 1e-4 and max(errs) < 1e-2
    assert O.rel_err(orc.E, z["it1_E"]) < 1e-4
    for ci in range(len(Y)):
        assert O.rel_err(Y[ci], z["it1_Y%d" % ci]) < 1e-3


# rtol of the trajectory: rec = sqrt(|X|^2 + |core|^2 - 2<X, core>) / |X| cancels ~45x at
# rec ~ 0.2, and the reference forms |core|^2 in fp32 with a 1.5e-5 relative error on c1
# (its chr1 value 1102.7616 against 1102.7785 exactly), so its own trajectory is off by
# ~1e-3 there.  The fp32 and fp64 restatements agree with each other to 2e-6.
@pytest.mark.parametrize("fixture,n_iter,rtol,conv,col", [
    ("als_small.npz", 4, 1e-4, False, False),
    ("c1_fit.npz", 10, 2e-3, False, False),
    ("als_conv_small.npz", 4, 1e-4, True, False),
    ("als_col_small.npz", 4, 1e-4, False, True),
    ("als_bad_small.npz", 4, 1e-4, False, False),
    ("als_badcol_small.npz", 4, 1e-4, False, True),
    ("als_defaults_small.npz", 4, 1e-4, True, False)])
def test_fit_trajectory_matches_reference(fixture, n_iter, rtol, conv, col):
    z = G.load(fixture)
    orc = _oracle_from(z, do_conv=conv, do_col=col)
    orc.fit(n_iter)
    traj = np.asarray(orc.rec_errors_total)
    np.testing.assert_allclose(traj, z["fit_rec_total"], rtol=rtol)
    n = len(orc.datas)
    A, B, D, E, _ = G.state(z, "fit", n)
    # the final embedding agrees after orthogonal Procrustes alignment
    assert O.rel_err(O.procrustes_align(orc.E, E), E) < 1e-3


@pytest.mark.parametrize("fixture,col", [("als_bad_small.npz", False), ("als_badcol_small.npz", True)])
def test_transform_with_bad_cells_matches_reference(fixture, col):
    """transform over good and bad-QC cells (parafac2_intergrative.py:742-834; 80 good and 16
    bad cells), after the 4-iteration fit: the embedding of all 96 cells against the
    reference's after orthogonal Procrustes alignment."""
    z = G.load(fixture)
    orc = _oracle_from(z, do_col=col)
    orc.fit(4)
    E = orc.transform(orc.U_last)
    ref = z["fit_E_transform"]
    assert E.shape == ref.shape == (96, int(z["rank"]))
    assert O.rel_err(O.procrustes_align(E, ref), ref) < 1e-3


def test_bad_cell_coverage_matches_reference_init():
    """bad_bin_cov of init_params (parafac2_intergrative.py:176-200, 268-271)."""
    z = G.load("als_badcol_small.npz")
    datas = G.chrom_datas(z, O)
    good = O.col_coverage(datas, np.float32)
    bad = O.col_coverage(datas, np.float32, bad=True)
    for k in range(len(datas)):
        for got, ref in ((good[k], z["init_bincov%d" % k]), (bad[k], z["init_badbincov%d" % k])):
            np.testing.assert_array_equal(np.isinf(got), np.isinf(ref))
            fin = np.isfinite(ref)
            assert O.rel_err(got[fin], ref[fin]) < 2e-6


@pytest.mark.parametrize("k,case", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_pack_matches_reference(k, case):
    """Input packing of raw per-cell matrices (FastHigashi_Wrapper.py:221-366): bin merging,
    the band, empty-bin removal and renumbering, coverage scaling, log1p and the clip."""
    z = G.load("pack.npz")
    n = int(z["n_cells"])
    cells = [(z["raw%d_cell%d" % (k, c)][0].astype(np.int64), z["raw%d_cell%d" % (k, c)][1].astype(np.int64),
              z["raw%d_val%d" % (k, c)]) for c in range(n)]
    merge, off_diag = (int(v) for v in z["out%d_%d_args" % (k, case)])
    idx, val, shape = O.pack_chromosome(cells, int(z["raw%d_nbin" % k]), z["reorder"], off_diag, merge)
    ref = "out%d_%d" % (k, case)
    assert tuple(shape) == tuple(z[ref + "_shape"])
    np.testing.assert_array_equal(idx, z[ref + "_idx"])
    np.testing.assert_array_equal(val, z[ref + "_val"])      # bit-exact: same fp32 operations


POST_KEYS = ["embed_all", "embed_raw", "embed_l2_norm", "embed_correct_coverage_fh",
             "embed_l2_norm_correct_coverage_fh", "embed_correct_batch",
             "embed_l2_norm_correct_batch"]


def postprocess_case(z, k):
    E = z["c%d_E" % k]
    Ds = [z["c%d_D%d" % (k, i)] for i in range(int(z["c%d_nD" % k]))]
    return E, Ds, z["c%d_readcount" % k], int(z["c%d_final_dim" % k]), z["c%d_reorder" % k]


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("restore", [False, True])
def test_postprocess_matches_reference(k, restore):
    """fetch_cell_embedding + correct_batch_linear (FastHigashi_Wrapper.py:750-878): the
    embedding, the quantile transform (bit for bit, ties included), the truncated SVDs with
    the reference's component signs, the regressions.  The reference's randomized fp32 SVD
    sits within 2e-5 of the exact one."""
    z = G.load("postprocess.npz")
    E, Ds, rc, fd, reorder = postprocess_case(z, k)
    st = O.fetch_cell_embedding(E, Ds, rc, fd, restore, reorder)
    O.correct_batch_linear(st, z["c%d_batch" % k], "batch", True, reorder)
    key = "c%d_r%d_" % (k, int(restore))
    np.testing.assert_array_equal(st["coverage_fh"], z[key + "coverage_fh"])
    for name in POST_KEYS:
        assert O.rel_err(st[name], z[key + name]) < 5e-5, name


def test_quantile_uniform_matches_published_transform_on_ties():
    """The restated quantile transform against scikit-learn's own, where it is installed,
    on heavy ties and sizes below and above the quantile count."""
    sk = pytest.importorskip("sklearn.preprocessing")
    rng = np.random.default_rng(5)
    for n in (1, 2, 7, 99, 100, 101, 2500):
        x = np.round(np.exp(rng.normal(8, 1.5, n)) / 50) * 50
        for nq in (100, 10):
            ref = sk.quantile_transform(x.reshape(-1, 1), n_quantiles=nq, copy=True)[:, 0]
            np.testing.assert_array_equal(O.quantile_uniform(x, nq), ref)


@pytest.mark.parametrize("conv", [False, True])
@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 2e-6)])
def test_only_partial_rwr_matches_reference(conv, dtype, tol):
    """only_partial_rwr (FastHigashi_Wrapper.py:569-655): auto-stopped walks per (bin batch,
    cell batch), good then bad-QC batches, placed and symmetrised; maps keyed by raw cell id."""
    z = G.load("impute.npz")
    datas = G.chrom_datas(z, O)
    for k, d in enumerate(datas):
        maps = O.only_partial_rwr(d, do_conv=conv, dtype=dtype)
        ref = z["conv%d_maps%d" % (int(conv), k)]
        assert tuple(z["conv%d_shape%d" % (int(conv), k)]) == (d.num_bin, d.num_bin)
        got = np.stack([maps[c] for c in range(ref.shape[0])])
        assert O.rel_err(got, ref) < tol


def test_multiresolution_fit_matches_reference():
    """res_list = [1 Mb, 500 kb] (parafac2_intergrative.py:558-590, 674-695): each chromosome's
    two datasets share B and D; its CP-ALS runs on their projected tensors stacked along the
    bins.  The trajectory, the per-dataset block errors and the fitted embedding."""
    z = G.load("als_multires_small.npz")
    datas = G.multires_datas(z, O)
    A, B, D, E, n_i = G.multires_state(z, "init")
    orc = O.ALSOracle(datas, int(z["rank"]), A, B, D, E, n_i).fit(int(z["n_iter"]))
    np.testing.assert_allclose(orc.rec_errors_total, z["fit_rec_total"], rtol=1e-4)
    np.testing.assert_allclose(np.stack(orc.rec_errors), z["fit_rec_block"], rtol=1e-4)
    _, _, _, Ef, _ = G.multires_state(z, "fit")
    assert O.rel_err(O.procrustes_align(orc.E, Ef), Ef) < 1e-3
