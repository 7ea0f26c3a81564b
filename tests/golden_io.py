"""Loaders for the golden fixtures under tests/golden (written by tests/golden/make_golden.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def coo_list(z, prefix="in"):
    out = []
    for k in range(int(z["n_chrom"])):
        idx = z["%s_idx%d" % (prefix, k)].astype(np.int32)
        val = z["%s_val%d" % (prefix, k)]
        shape = tuple(int(s) for s in z["%s_shape%d" % (prefix, k)])
        out.append((idx, val, shape))
    return out


def chrom_datas(z, oracle_mod, names=None):
    coo = coo_list(z)
    bs_bin = np.broadcast_to(np.asarray(z["bs_bin"]), (len(coo),))
    bs_cell = np.broadcast_to(np.asarray(z["bs_cell"]), (len(coo),))
    names = names or ["chr%d" % (k + 1) for k in range(len(coo))]
    out = []
    good = int(z["good_qc_num"]) if "good_qc_num" in z else -1
    for k, (idx, val, shape) in enumerate(coo):
        n_good = shape[2] if good < 0 else good
        out.append(oracle_mod.ChromData(names[k], idx, val, shape[0], n_good, int(bs_bin[k]),
                                        int(bs_cell[k]), int(z["flank"]), shape[2]))
    return out


def state(z, prefix, n_chrom, names=None):
    names = names or ["chr%d" % (k + 1) for k in range(n_chrom)]
    A = [z["%s_A%d" % (prefix, k)] for k in range(n_chrom)]
    B = {names[k]: z["%s_B%d" % (prefix, k)] for k in range(n_chrom)}
    D = {names[k]: z["%s_D%d" % (prefix, k)] for k in range(n_chrom)}
    return A, B, D, z["%s_E" % prefix], z["%s_n_i" % prefix]


def multires_datas(z, oracle_mod):
    """The oracle's datasets of a multi-resolution fixture: one per (chromosome, resolution),
    named by chromosome, in the fixture's dataset order."""
    coo = coo_list(z)
    names = [str(s) for s in z["names"]]
    good = int(z["good_qc_num"]) if "good_qc_num" in z else -1
    out = []
    for k, (idx, val, shape) in enumerate(coo):
        n_good = shape[2] if good < 0 else good
        out.append(oracle_mod.ChromData(names[k], idx, val, shape[0], n_good, int(z["bs_bin"]),
                                        int(z["bs_cell"]), int(z["flank"]), shape[2]))
    return out


def multires_state(z, prefix):
    """(A per dataset, B and D per chromosome, E, n_i per dataset) of a multi-resolution
    fixture."""
    names = [str(s) for s in z["names"]]
    chroms = list(dict.fromkeys(names))
    A = [z["%s_A%d" % (prefix, k)] for k in range(len(names))]
    B = {c: z["%s_B%d" % (prefix, i)] for i, c in enumerate(chroms)}
    D = {c: z["%s_D%d" % (prefix, i)] for i, c in enumerate(chroms)}
    return A, B, D, z["%s_E" % prefix], z["%s_n_i" % prefix]
