"""Quality of the GPU init_params (fh_gb300/init.py) against the reference's own init.

The reference's init (parafac2_intergrative.py:61-301) draws its features through
scikit-learn's unseeded randomized TruncatedSVD, so no run reproduces it; the GPU init
computes the same quantities (auto-stopped walk epochs n_i, band features, their truncated SVD,
E and D) with its own random sketch.  What a user needs is that a fit from it is as good: over
several seeds, the fit's final reconstruction error is within 1 % of the reference's fit from
the reference's init (the fixtures' trajectories), and the walk epochs n_i are the reference's.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import golden_io as G
from gpu_util import datasets_from

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fixture,n_iter", [("c1_fit.npz", 10), ("als_small.npz", 4)])
def test_fit_from_gpu_init_reaches_reference_loss(fixture, n_iter):
    from fh_gb300 import Fast_Higashi_core
    z = G.load(fixture)
    ds = datasets_from(z)
    ref_final = float(z["fit_rec_total"][-1])
    finals = []
    for seed in (0, 1, 2):
        m = Fast_Higashi_core(int(z["rank"]), int(z["flank"]), [int(z["resolution"])]).to("cuda")
        m._sizes(ds, float(z["dim1"]), None)
        m.init_params(ds, False, True, False, seed=seed)
        np.testing.assert_array_equal(np.asarray(m.n_i), z["init_n_i"])
        m.fit(ds, size_ratio=float(z["dim1"]), n_iter_max=n_iter, n_iter_parafac=1,
              do_conv=False, do_rwr=True, do_col=False, tol=0, run_init=False, verbose=False)
        finals.append(float(m.rec_errors_total[-1]))
    print(fixture, "final loss from the GPU init (seeds 0-2):", finals,
          "reference's fit from its own init:", ref_final)
    assert max(finals) <= 1.01 * ref_final


def test_multiresolution_fit_from_gpu_init_reaches_reference_loss():
    """The two-resolution fixture (1 Mb and 500 kb datasets of each chromosome): the 500 kb
    features go through the 1 Mb pooling (ll = 2) and each chromosome's features span both
    resolutions, as the reference's init builds them."""
    from fh_gb300 import Fast_Higashi_core
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    z = G.load("als_multires_small.npz")
    names = [str(s) for s in z["names"]]
    ds = [Chrom_Dataset(Sparse(idx, val, shape), int(z["bs_bin"]), int(z["bs_cell"]),
                        compact=True, flank=int(z["flank"]), chrom=names[k],
                        resolution=int(z["res"][k]))
          for k, (idx, val, shape) in enumerate(G.coo_list(z))]
    res_list = sorted(set(int(r) for r in z["res"]), reverse=True)
    ref_final = float(z["fit_rec_total"][-1])
    finals = []
    for seed in (0, 1, 2):
        m = Fast_Higashi_core(int(z["rank"]), int(z["flank"]), res_list).to("cuda")
        m._sizes(ds, float(z["dim1"]), None)
        m.init_params(ds, False, True, False, seed=seed)
        np.testing.assert_array_equal(np.asarray(m.n_i), z["init_n_i"])
        m.fit(ds, size_ratio=float(z["dim1"]), n_iter_max=int(z["n_iter"]), n_iter_parafac=1,
              do_conv=False, do_rwr=True, do_col=False, tol=0, run_init=False, verbose=False)
        finals.append(float(m.rec_errors_total[-1]))
    print("multi-resolution: final loss from the GPU init (seeds 0-2):", finals,
          "reference's fit from its own init:", ref_final)
    assert max(finals) <= 1.01 * ref_final
