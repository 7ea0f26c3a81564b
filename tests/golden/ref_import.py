"""Imports the reference Fast-Higashi hot path in this container (fixture generation only).

Two host-side shims, both outside the arithmetic:
  1. ``fasthigashi/util.py:2`` imports pandas, which is not installed; a stub module
     stands in during the import and is removed right after (a stub left in
     ``sys.modules`` breaks scikit-learn's optional-pandas probes).
  2. ``Sparse.__init__`` (``fasthigashi/sparse_for_schic.py:63-66``) calls
     ``np.array(shape, copy=False)``, which NumPy 2 rejects for tuples; the
     objects are built with ``copy=True`` (same values).
``import_wrapper`` also stubs h5py (not installed; the packing path never calls it) while
``fasthigashi/FastHigashi_Wrapper.py`` imports.
Only ``tests/golden/make_golden.py`` uses this module; nothing that runs on a
GPU host does.
"""
import os
import sys
import types

# the checkout of the reference project (the folder that holds fasthigashi/), named by the
# caller: fixture generation has no default location
REF_ROOT = os.environ.get("FH_REFERENCE_ROOT", "")


def _root():
    if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "fasthigashi")):
        raise RuntimeError("set FH_REFERENCE_ROOT to a checkout of the reference project "
                           "(the folder holding fasthigashi/)")
    return REF_ROOT


def import_reference():
    root = _root()
    if root not in sys.path:
        sys.path.insert(0, root)
    had_pd = "pandas" in sys.modules
    if not had_pd:
        sys.modules["pandas"] = types.ModuleType("pandas")
    try:
        import fasthigashi.parafac2_intergrative as p2
        import fasthigashi.parafac_integrative as p1
        import fasthigashi.partial_rwr as prwr
        import fasthigashi.project2orthogonal as p2o
        import fasthigashi.sparse_for_schic as sfs
    finally:
        if not had_pd:
            del sys.modules["pandas"]
    # quiet progress printing of the reference's tqdm bars
    return dict(core=p2, parafac=p1, rwr=prwr, p2o=p2o, sparse=sfs)


def import_wrapper():
    """fasthigashi.FastHigashi_Wrapper with pandas and h5py stubbed during its import."""
    root = _root()
    if root not in sys.path:
        sys.path.insert(0, root)
    stubs = [m for m in ("pandas", "h5py") if m not in sys.modules]
    for m in stubs:
        sys.modules[m] = types.ModuleType(m)
    try:
        import fasthigashi.FastHigashi_Wrapper as wr
    finally:
        for m in stubs:
            del sys.modules[m]
    return wr


def build_chrom_datasets(ref, coo_list, names, bs_bins, bs_cells, flank, resolution,
                         good_qc_num=-1):
    sfs = ref["sparse"]
    out = []
    for (idx, vals, shape), name, bsb, bsc in zip(coo_list, names, bs_bins, bs_cells):
        obj = sfs.Sparse(idx.copy(), vals.copy(), shape, copy=True)
        obj.sort_indices()
        ds = sfs.Chrom_Dataset(tensor=obj, bs_bin=bsb, bs_cell=bsc, good_qc_num=good_qc_num,
                               kind='hic', upper_sim=False, compact=True, flank=flank,
                               chrom=name, resolution=resolution)
        out.append(ds)
    return out
