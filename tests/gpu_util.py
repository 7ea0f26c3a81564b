"""Helpers shared by the GPU tests."""
import numpy as np

from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
import golden_io as G


def datasets_from(z, names=None, resolution=None):
    coo = G.coo_list(z)
    n = len(coo)
    bs_bin = np.broadcast_to(np.asarray(z["bs_bin"]), (n,))
    bs_cell = np.broadcast_to(np.asarray(z["bs_cell"]), (n,))
    names = names or ["chr%d" % (k + 1) for k in range(n)]
    res = int(z["resolution"]) if resolution is None and "resolution" in z else (resolution or 1000000)
    good = int(z["good_qc_num"]) if "good_qc_num" in z else -1
    out = []
    for k, (idx, val, shape) in enumerate(coo):
        out.append(Chrom_Dataset(Sparse(idx, val, shape), int(bs_bin[k]), int(bs_cell[k]),
                                 good_qc_num=good, compact=True, flank=int(z["flank"]),
                                 chrom=names[k], resolution=res))
    return out
