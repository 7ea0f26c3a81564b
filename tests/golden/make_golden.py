"""Generates the golden fixtures by running the reference Fast-Higashi in this container.

    python tests/golden/make_golden.py          (needs the reference tree; CPU only)

Every output is produced by the reference's own functions on seeded synthetic inputs
(``fh_gb300.synth``), in float32 on the CPU, with the two import shims described in
``ref_import.py``.  Fixtures:

  rwr_tiles.npz    every (bin batch, cell batch) tile of the ``tiny`` workload with
                   bs_bin=12, bs_cell=10, flank=4: the densified input from
                   ``Chrom_Dataset.fetch`` and ``partial_rwr`` outputs with
                   force_rwr_epochs=3 and with the auto-stop rule (plus its epoch count).
  parafac.npz      ``parafac`` on a random 3-way tensor for n_iter_max 1 and 3.
  als_small.npz    the ``small`` workload with bs_bin=25, bs_cell=40: the state after
                   ``init_params``, one ``update_meta_embedding_interactions`` call from it,
                   and a 4-iteration ``fit`` from the same state (loss trajectory,
                   factors, ``transform`` embedding).
  c1_fit.npz       the 200-cell, 3-chromosome, R=16, band 10 workload with the reference's
                   GPU batching: the input, the initial state, the 10-iteration loss
                   trajectory and the final factors and embedding.
  rwr_conv_tiles.npz  the tiles of rwr_tiles.npz through partial_rwr with do_conv=True (the
                   3 x 3 mean before the walk): force_rwr_epochs=3, the auto-stop rule, and
                   do_rwr=False (the smoothed tile alone).
  als_conv_small.npz  als_small.npz's workload fitted with do_conv=True.
  rwr_col_tiles.npz  the tiles of rwr_tiles.npz through partial_rwr with do_col=True and a
                   seeded coverage argument (positive, a few entries inf): force_rwr_epochs=3,
                   the auto-stop rule, and do_conv=True with force_rwr_epochs=3.
  als_col_small.npz  als_small.npz's workload fitted with do_col=True, with the coverage
                   rows (bin_cov_list) init_params computed.
  pack.npz         FastHigashi.pack_training_data_one_process (FastHigashi_Wrapper.py:221-366)
                   on seeded raw per-cell contact matrices of two chromosomes (some bins empty in
                   every cell, contacts past the band, a cell order to apply), with merge
                   factors 1 and 2: the packed (row, col, cell) indices, values and shape.
  als_multires_small.npz  the small workload's chromosomes at 1 Mb and at 500 kb under the same
                   names, fitted with res_list=[1 Mb, 500 kb] (B and D shared per chromosome):
                   init, trajectory, final state, transform.
  impute.npz       FastHigashi.only_partial_rwr (FastHigashi_Wrapper.py:569-655): every
                   cell's imputed map of the tiny workload (12-row bin batches, cell batches
                   of 10, 6 bad-QC cells, a cell order), with and without do_conv.
  postprocess.npz  FastHigashi.fetch_cell_embedding and correct_batch_linear
                   (FastHigashi_Wrapper.py:750-878): the concatenated embedding, its truncated
                   SVD and row-normalised form, the quantile-transformed read counts, the
                   coverage-regressed and label-regressed embeddings, with and without the
                   restored cell order, for als_small.npz's fitted factors and seeded ones.
  als_defaults_small.npz  the same workload with the reference's fit defaults (do_conv=True,
                   do_rwr=False: the 3 x 3 mean and no walk).
  als_bad_small.npz / als_badcol_small.npz  the same workload with its last 16 cells bad-QC
                   (good_qc_num=80): init, fit and transform (which embeds the bad cells too),
                   with do_col=False / True (the latter with bin_cov and bad_bin_cov).

    FH_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py \
        rwr_conv als_conv rwr_col als_col als_bad als_defaults pack postprocess impute multires
"""
import copy
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", "..", "fast-higashi_gb300"))

from ref_import import import_reference, import_wrapper, build_chrom_datasets  # noqa: E402
from fh_gb300 import synth  # noqa: E402

torch.set_num_threads(4)
ref = import_reference()
core = ref["core"]
CPU = torch.device("cpu")


def coo_arrays(prefix, coo):
    out = {}
    for k, (idx, vals, shape) in enumerate(coo):
        # rows, columns and cells of these workloads fit int16; the loaders widen them
        out["%s_idx%d" % (prefix, k)] = idx.astype(np.int16)
        out["%s_val%d" % (prefix, k)] = vals.astype(np.float32)
        out["%s_shape%d" % (prefix, k)] = np.asarray(shape, dtype=np.int64)
    return out


def make_rwr_tiles():
    w = synth.workload("tiny")
    coo, _ = synth.generate(w, seed=11)
    ds = build_chrom_datasets(ref, coo, w.chrom_names, [12] * 2, [10] * 2, w.band, w.resolution)
    out = coo_arrays("in", coo)
    out.update(bs_bin=12, bs_cell=10, flank=w.band, n_chrom=len(coo))
    k = 0
    for ci, d in enumerate(ds):
        for bi in range(d.num_bin_batch):
            loc = d.local_bin_slice_list[bi]
            for cj in range(d.num_cell_batch):
                (x, _), kind = d.fetch(bi, cj, save_context=dict(device=CPU), transpose=True)
                y3, _ = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, False, True, False,
                                               force_rwr_epochs=3, return_rwr_iter=True)
                ya, na = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, False, True, False,
                                                force_rwr_epochs=-1, return_rwr_iter=True,
                                                final_transpose=False)
                out["t%d_meta" % k] = np.array([ci, bi, cj, loc.start, loc.stop, na], dtype=np.int64)
                out["t%d_x" % k] = x.numpy()
                out["t%d_y3" % k] = y3.contiguous().numpy()
                out["t%d_yauto" % k] = ya.contiguous().numpy()
                k += 1
    out["n_tiles"] = k
    np.savez_compressed(os.path.join(HERE, "rwr_tiles.npz"), **out)
    print("rwr_tiles", k, "tiles")


def make_rwr_conv_tiles():
    w = synth.workload("tiny")
    coo, _ = synth.generate(w, seed=11)
    ds = build_chrom_datasets(ref, coo, w.chrom_names, [12] * 2, [10] * 2, w.band, w.resolution)
    out = coo_arrays("in", coo)
    out.update(bs_bin=12, bs_cell=10, flank=w.band, n_chrom=len(coo))
    k = 0
    for ci, d in enumerate(ds):
        for bi in range(d.num_bin_batch):
            loc = d.local_bin_slice_list[bi]
            for cj in range(d.num_cell_batch):
                (x, _), kind = d.fetch(bi, cj, save_context=dict(device=CPU), transpose=True)
                y3, _ = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, True, True, False,
                                               force_rwr_epochs=3, return_rwr_iter=True)
                ya, na = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, True, True, False,
                                                force_rwr_epochs=-1, return_rwr_iter=True,
                                                final_transpose=False)
                y0, _ = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, True, False, False,
                                               return_rwr_iter=True)
                out["t%d_meta" % k] = np.array([ci, bi, cj, loc.start, loc.stop, na], dtype=np.int64)
                out["t%d_x" % k] = x.numpy()
                out["t%d_y3" % k] = y3.contiguous().numpy()
                out["t%d_yauto" % k] = ya.contiguous().numpy()
                out["t%d_y0" % k] = y0.contiguous().numpy()
                k += 1
    out["n_tiles"] = k
    np.savez_compressed(os.path.join(HERE, "rwr_conv_tiles.npz"), **out)
    print("rwr_conv_tiles", k, "tiles")


def make_rwr_col_tiles():
    w = synth.workload("tiny")
    coo, _ = synth.generate(w, seed=11)
    ds = build_chrom_datasets(ref, coo, w.chrom_names, [12] * 2, [10] * 2, w.band, w.resolution)
    rng = np.random.default_rng(17)
    out = coo_arrays("in", coo)
    out.update(bs_bin=12, bs_cell=10, flank=w.band, n_chrom=len(coo))
    k = 0
    for ci, d in enumerate(ds):
        for bi in range(d.num_bin_batch):
            loc = d.local_bin_slice_list[bi]
            for cj in range(d.num_cell_batch):
                (x, _), kind = d.fetch(bi, cj, save_context=dict(device=CPU), transpose=True)
                cov = rng.uniform(0.5, 4.0, size=(x.shape[0], x.shape[2])).astype(np.float32)
                cov[rng.random(cov.shape) < 0.05] = np.inf
                tc = torch.from_numpy(cov)
                y3, _ = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, False, True, True,
                                               bin_cov=tc.clone(), force_rwr_epochs=3,
                                               return_rwr_iter=True)
                ya, na = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, False, True, True,
                                                bin_cov=tc.clone(), force_rwr_epochs=-1,
                                                return_rwr_iter=True, final_transpose=False)
                yc, _ = ref["rwr"].partial_rwr(x.clone(), loc.start, loc.stop, True, True, True,
                                               bin_cov=tc.clone(), force_rwr_epochs=3,
                                               return_rwr_iter=True)
                out["t%d_meta" % k] = np.array([ci, bi, cj, loc.start, loc.stop, na], dtype=np.int64)
                out["t%d_x" % k] = x.numpy()
                out["t%d_cov" % k] = cov
                out["t%d_y3" % k] = y3.contiguous().numpy()
                out["t%d_yauto" % k] = ya.contiguous().numpy()
                out["t%d_yconv3" % k] = yc.contiguous().numpy()
                k += 1
    out["n_tiles"] = k
    np.savez_compressed(os.path.join(HERE, "rwr_col_tiles.npz"), **out)
    print("rwr_col_tiles", k, "tiles")


def pack_raw_cells(rng, nbin, n_cells, reach=12, empty=()):
    """Seeded raw per-cell contact matrices (scipy csr, float32, both triangles)."""
    from scipy.sparse import coo_matrix
    out = []
    for _ in range(n_cells):
        i, j = np.triu_indices(nbin)
        keep = (j - i) <= reach
        i, j = i[keep], j[keep]
        lam = 3.0 * (j - i + 1.0) ** -1.1 * rng.uniform(0.3, 1.5)
        c = rng.poisson(lam).astype(np.float32)
        for e in empty:
            c[(i == e) | (j == e)] = 0
        nz = c > 0
        i, j, c = i[nz], j[nz], c[nz]
        off = i != j
        rows = np.concatenate([i, j[off]])
        cols = np.concatenate([j, i[off]])
        vals = np.concatenate([c, c[off]])
        out.append(coo_matrix((vals, (rows, cols)), shape=(nbin, nbin)).tocsr())
    return out


def make_pack():
    import tempfile
    import types as T
    wr = import_wrapper()
    rng = np.random.default_rng(21)
    chroms = [("chrA", 40, (5, 17)), ("chrB", 33, (0, 32))]
    n_cells = 24
    reorder = rng.permutation(n_cells)
    out = dict(reorder=reorder, n_cells=n_cells, n_chrom=len(chroms))
    with tempfile.TemporaryDirectory() as raw:
        for k, (name, nbin, empty) in enumerate(chroms):
            mats = pack_raw_cells(rng, nbin, n_cells, empty=empty)
            arr = np.empty(n_cells, dtype=object)
            for c, m in enumerate(mats):
                arr[c] = m
                cm = m.tocoo()
                out["raw%d_cell%d" % (k, c)] = np.stack([cm.row, cm.col]).astype(np.int32)
                out["raw%d_val%d" % (k, c)] = cm.data.astype(np.float32)
            out["raw%d_nbin" % k] = nbin
            np.save(os.path.join(raw, "%s_sparse_adj.npy" % name), arr, allow_pickle=True)
            for case, (merge, off_diag) in enumerate(((1, 4), (2, 3))):
                me = T.SimpleNamespace(config={}, temp_dir=os.path.join(raw, "none"),
                                       sum_sparse_coo=wr.FastHigashi.sum_sparse_coo)
                idx, val, shape = wr.FastHigashi.pack_training_data_one_process(
                    me, raw, name, reorder, off_diag=off_diag, fac_size=1, merge_fac_row=merge,
                    merge_fac_col=merge, is_sym=True, filename_pattern="%s_sparse_adj.npy",
                    force_shift=False, batch_norm=True, bar=None)
                key = "out%d_%d" % (k, case)
                out[key + "_idx"] = idx
                out[key + "_val"] = val
                out[key + "_shape"] = np.asarray(shape, dtype=np.int64)
                out[key + "_args"] = np.asarray([merge, off_diag], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "pack.npz"), **out)
    print("pack", {k: v.shape for k, v in out.items() if k.startswith("out") and k.endswith("_idx")})


def make_postprocess():
    """FastHigashi.fetch_cell_embedding and correct_batch_linear (FastHigashi_Wrapper.py:
    750-878) on (0) the fitted factors of als_small.npz and (1) seeded factors of 300 cells,
    R = 16, four chromosomes of rank 12; coverage regression inside fetch_cell_embedding, then
    a three-level categorical label with the intercept added back.  TruncatedSVD draws from
    NumPy's global generator, seeded before each call."""
    import types as T
    wr = import_wrapper()
    z = np.load(os.path.join(HERE, "als_small.npz"))
    rng = np.random.default_rng(31)
    cases = [(z["fit_E"].astype(np.float32), [z["fit_D%d" % i].astype(np.float32)
                                               for i in range(3)], 8, None)]
    C, R = 300, 16
    E = rng.standard_normal((C, R)).astype(np.float32) * np.linspace(3, 0.5, R)[None]
    Ds = [(rng.standard_normal((R, 12)) * rng.uniform(0.5, 2, 12)[None]).astype(np.float32)
          for _ in range(4)]
    cases.append((E, Ds, R, 12))
    out = dict(n_case=len(cases))
    for k, (E, Ds, rank, final_dim) in enumerate(cases):
        C = E.shape[0]
        readcount = np.round(np.exp(rng.normal(10, 0.8, C))).astype(np.int64)
        readcount[:3] = readcount[3]                 # ties among the quantiles' inputs
        batch = np.array(["b%d" % v for v in rng.integers(0, 3, C)])
        reorder = rng.permutation(C)
        for restore in (False, True):
            me = T.SimpleNamespace(rank=rank, D_list=Ds, meta_embedding=E,
                                   coverage_feats=readcount.reshape((-1, 1)),
                                   label_info={"batch": batch}, reorder=reorder,
                                   embedding_storage=None)
            me.restore_order_fun = lambda x, me=me: wr.FastHigashi.restore_order_fun(me, x)
            me.correct_batch_linear = (lambda name, back, me=me:
                                       wr.FastHigashi.correct_batch_linear(me, name, back))
            np.random.seed(100 + k)
            store = wr.FastHigashi.fetch_cell_embedding(me, final_dim=final_dim,
                                                        restore_order=restore)
            np.random.seed(200 + k)
            wr.FastHigashi.correct_batch_linear(me, "batch", True)
            key = "c%d_r%d_" % (k, int(restore))
            for name, v in store.items():
                if isinstance(v, np.ndarray):
                    out[key + name] = v
            out[key + "coverage_fh"] = np.asarray(me.label_info["coverage_fh"])
        out["c%d_E" % k] = E
        out["c%d_nD" % k] = len(Ds)
        for i, D in enumerate(Ds):
            out["c%d_D%d" % (k, i)] = D
        out["c%d_readcount" % k] = readcount
        out["c%d_batch" % k] = batch
        out["c%d_reorder" % k] = reorder
        out["c%d_final_dim" % k] = rank if final_dim is None else final_dim
    np.savez_compressed(os.path.join(HERE, "postprocess.npz"), **out)
    print("postprocess", sorted(k for k in out if k.startswith("c1_r0")))


def make_impute():
    """FastHigashi.only_partial_rwr (FastHigashi_Wrapper.py:569-655) on the tiny workload with
    12-row bin batches, cell batches of 10 and its last 6 cells bad-QC, without and with
    do_conv; h5py is replaced by an in-memory recorder of the datasets it is asked to write."""
    import types as T
    wr = import_wrapper()
    w = synth.workload("tiny")
    coo, _ = synth.generate(w, seed=4)
    good = w.n_cells - 6
    reorder = np.random.default_rng(9).permutation(w.n_cells)
    out = coo_arrays("in", coo)
    out.update(n_chrom=len(coo), bs_bin=12, bs_cell=10, flank=w.band, good_qc_num=good,
               resolution=w.resolution, reorder=reorder)

    class Group(dict):
        def create_dataset(self, name, data):
            self[name] = np.asarray(data)

    class File(dict):
        def __init__(self, path, mode):
            super().__init__()

        def create_group(self, name):
            g = self[name] = Group()
            return g

        def close(self):
            pass

    files = []
    fake = T.ModuleType("h5py")
    fake.File = lambda path, mode: files.append(File(path, mode)) or files[-1]
    wr.h5py = fake
    for conv in (False, True):
        ds = build_chrom_datasets(ref, coo, w.chrom_names, [12] * len(coo), [10] * len(coo),
                                  w.band, w.resolution, good_qc_num=good)
        me = T.SimpleNamespace(all_matrix=ds, chrom_list=w.chrom_names, path2result_dir=HERE,
                               do_conv=conv, do_rwr=True, device=CPU, reorder=reorder)
        wr.FastHigashi.only_partial_rwr(me)
        f = files[-1]
        for k, name in enumerate(w.chrom_names):
            g = f[name]
            out["conv%d_shape%d" % (int(conv), k)] = g["shape"]
            out["conv%d_maps%d" % (int(conv), k)] = np.stack([g[str(int(reorder[c]))]
                                                              for c in range(w.n_cells)])
    np.savez_compressed(os.path.join(HERE, "impute.npz"), **out)
    print("impute", {k: v.shape for k, v in out.items() if "maps" in k})


def make_multires():
    """als_multires_small.npz: the small workload's three chromosomes at 1 Mb and, under the
    same names, an independent draw at 500 kb (twice the bins), fitted together with
    res_list=[1 Mb, 500 kb]: six datasets, B and D shared by the two resolutions of a
    chromosome.  The reference's init, its 4-iteration trajectory and final state, and
    transform's embedding."""
    import dataclasses
    w1 = synth.workload("small")
    w2 = dataclasses.replace(w1, name="small500", chrom_bins=[2 * b for b in w1.chrom_bins],
                             resolution=500_000, chrom_names=list(w1.chrom_names))
    coo1, _ = synth.generate(w1, seed=3)
    coo2, _ = synth.generate(w2, seed=4)
    n = len(coo1)
    ds = (build_chrom_datasets(ref, coo1, w1.chrom_names, [25] * n, [40] * n, w1.band,
                               w1.resolution) +
          build_chrom_datasets(ref, coo2, w2.chrom_names, [25] * n, [40] * n, w2.band,
                               w2.resolution))
    res_list = [w1.resolution, w2.resolution]
    np.random.seed(5)
    torch.manual_seed(5)
    m = core.Fast_Higashi_core(rank=w1.rank, off_diag=w1.band, res_list=res_list).to(CPU)
    m.fit(ds, size_ratio=w1.dim1, n_iter_max=0, n_iter_parafac=1, do_conv=False, do_rwr=True,
          do_col=False, tol=0, run_init=True)
    st0 = snapshot(m)
    out = coo_arrays("in", coo1 + coo2)
    out.update(state_arrays("init", st0, w1.chrom_names))
    out.update(n_chrom=2 * n, names=np.asarray(w1.chrom_names + w2.chrom_names),
               res=np.asarray([w1.resolution] * n + [w2.resolution] * n, dtype=np.int64),
               bs_bin=25, bs_cell=40, flank=w1.band, rank=w1.rank, dim1=w1.dim1, n_iter=4,
               sizes=np.asarray([m.chrom2size[c] for c in w1.chrom_names]))
    m2 = core.Fast_Higashi_core(rank=w1.rank, off_diag=w1.band, res_list=res_list).to(CPU)
    inject(m2, st0)
    with FitLocals() as fl:
        m2.fit(ds, size_ratio=w1.dim1, n_iter_max=4, n_iter_parafac=1, do_conv=False,
               do_rwr=True, do_col=False, tol=0, run_init=False)
    res = m2.transform(ds, False, True, False)
    out["fit_rec_total"] = np.asarray(fl.locals["rec_errors_total"], dtype=np.float64)
    out["fit_rec_block"] = np.stack([np.asarray(x).ravel() for x in fl.locals["rec_errors"]])
    out.update(state_arrays("fit", snapshot(m2), w1.chrom_names))
    out["fit_E_transform"] = res[1][3].numpy()
    np.savez_compressed(os.path.join(HERE, "als_multires_small.npz"), **out)
    print("multires rec trajectory", out["fit_rec_total"], "blocks", out["fit_rec_block"].shape)


def make_parafac():
    rng = np.random.default_rng(5)
    X = rng.standard_normal((40, 6, 9)).astype(np.float32)
    init = [1 + 0.01 * rng.standard_normal((40, 6)), np.eye(6) + 0.01 * rng.standard_normal((6, 6)),
            rng.standard_normal((9, 6))]
    init = [a.astype(np.float32) for a in init]
    out = dict(X=X, A0=init[0], B0=init[1], D0=init[2])
    for n in (1, 3):
        f, ln, lx = ref["parafac"].parafac(torch.from_numpy(X), rank=6, n_iter_max=n,
                                           init=[torch.from_numpy(a.copy()) for a in init])
        out["A%d" % n], out["B%d" % n], out["D%d" % n] = [t.numpy() for t in f]
        out["ln%d" % n], out["lx%d" % n] = ln, lx
    np.savez_compressed(os.path.join(HERE, "parafac.npz"), **out)
    print("parafac")


class FitLocals:
    """Captures the local loss lists of Fast_Higashi_core.fit when it returns."""

    def __init__(self):
        self.locals = None

    def __enter__(self):
        def prof(frame, event, arg):
            if event == "return" and frame.f_code is core.Fast_Higashi_core.fit.__code__:
                self.locals = dict(frame.f_locals)
        sys.setprofile(prof)
        return self

    def __exit__(self, *a):
        sys.setprofile(None)


def snapshot(model):
    return dict(A=[a.clone() for a in model.A_list],
                B={k: v.clone() for k, v in model.B_dict.items()},
                D={k: v.clone() for k, v in model.D_dict.items()},
                E=model.meta_embedding.clone(), n_i=np.array(model.n_i).copy(),
                bin_cov=[b.clone() for b in model.bin_cov_list],
                bad_bin_cov=copy.deepcopy(model.bad_bin_cov_list))


def inject(model, st):
    model.A_list = [a.clone() for a in st["A"]]
    model.B_dict = {k: v.clone() for k, v in st["B"].items()}
    model.D_dict = {k: v.clone() for k, v in st["D"].items()}
    model.meta_embedding = st["E"].clone()
    model.n_i = st["n_i"].copy()
    model.bin_cov_list = [b.clone() for b in st["bin_cov"]]
    model.bad_bin_cov_list = copy.deepcopy(st["bad_bin_cov"])


def state_arrays(prefix, st, names):
    out = {"%s_E" % prefix: st["E"].numpy(), "%s_n_i" % prefix: np.asarray(st["n_i"])}
    for k, a in enumerate(st["A"]):
        out["%s_A%d" % (prefix, k)] = a.numpy()
    for k, n in enumerate(names):
        out["%s_B%d" % (prefix, k)] = st["B"][n].numpy()
        out["%s_D%d" % (prefix, k)] = st["D"][n].numpy()
    return out


def run_fit(w, ds, n_iter, init_state, dim1, do_conv=False, do_col=False, do_rwr=True):
    m = core.Fast_Higashi_core(rank=w.rank, off_diag=w.band, res_list=[w.resolution]).to(CPU)
    inject(m, init_state)
    with FitLocals() as fl:
        m.fit(ds, size_ratio=dim1, n_iter_max=n_iter, n_iter_parafac=1, do_conv=do_conv,
              do_rwr=do_rwr, do_col=do_col, tol=0, run_init=False)
    res = m.transform(ds, do_conv, do_rwr, do_col)
    return m, fl.locals, res


def make_als(name, wname, bs_bin, bs_cell, n_iter, seed, save_input=True, save_U=True,
             do_conv=False, do_col=False, good_qc_num=-1, do_rwr=True):
    w = synth.workload(wname)
    coo, _ = synth.generate(w, seed=seed)
    bsb = [bs_bin or synth.recommend_batches(w, nb, w.n_cells)[0] for nb in w.chrom_bins]
    bsc = [bs_cell or w.n_cells for _ in w.chrom_bins]
    ds = build_chrom_datasets(ref, coo, w.chrom_names, bsb, bsc, w.band, w.resolution,
                              good_qc_num=good_qc_num)
    np.random.seed(seed)
    torch.manual_seed(seed)
    m = core.Fast_Higashi_core(rank=w.rank, off_diag=w.band, res_list=[w.resolution]).to(CPU)
    m.fit(ds, size_ratio=w.dim1, n_iter_max=0, n_iter_parafac=1, do_conv=do_conv, do_rwr=do_rwr,
          do_col=do_col, tol=0, run_init=True)
    st0 = snapshot(m)
    out = coo_arrays("in", coo) if save_input else {}
    out.update(state_arrays("init", st0, w.chrom_names))
    if do_col:
        for k, c in enumerate(st0["bin_cov"]):
            out["init_bincov%d" % k] = c.numpy()
        for k, c in enumerate(st0["bad_bin_cov"]):
            if torch.is_tensor(c):
                out["init_badbincov%d" % k] = c.numpy()
    if good_qc_num >= 0:
        out["good_qc_num"] = good_qc_num
    out["do_rwr"] = int(do_rwr)
    out.update(bs_bin=np.asarray(bsb), bs_cell=np.asarray(bsc), flank=w.band, rank=w.rank,
               resolution=w.resolution, dim1=w.dim1, n_iter=n_iter, seed=seed,
               n_chrom=len(coo), sizes=np.asarray([m.chrom2size[n] for n in w.chrom_names]))
    # one update_meta_embedding_interactions call from the initial state
    proj_list = [[torch.empty(0)] * d.num_bin_batch for d in ds]
    ptl = {d.chrom: torch.empty([d.num_bin, m.chrom2size[d.chrom], w.rank]) for d in ds}
    r = m.update_meta_embedding_interactions(ds, proj_list, ptl, do_conv=do_conv, do_rwr=do_rwr,
                                             do_col=do_col, first_iter=True)
    pl, ptl, exU, exV, tn = r
    for ci, d in enumerate(ds):
        for bi in range(d.num_bin_batch if save_U else 0):
            out["it1_U%d_%d" % (ci, bi)] = pl[ci][bi].numpy()
        out["it1_Y%d" % ci] = ptl[d.chrom].numpy()
    out.update(it1_exU=np.asarray(exU).ravel(), it1_exV=float(exV), it1_tnorm=np.asarray(tn).ravel(),
               it1_E=m.meta_embedding.numpy())
    # the fit loop from the same state
    m2, loc, res = run_fit(w, ds, n_iter, st0, w.dim1, do_conv, do_col, do_rwr)
    out["fit_rec_total"] = np.asarray(loc["rec_errors_total"], dtype=np.float64)
    out["fit_rec_block"] = np.stack([np.asarray(x).ravel() for x in loc["rec_errors"]])
    out.update(state_arrays("fit", snapshot(m2), w.chrom_names))
    out["fit_E_transform"] = res[1][3].numpy()
    m3, loc1, _ = run_fit(w, ds, 1, st0, w.dim1, do_conv, do_col, do_rwr)
    out.update(state_arrays("one", snapshot(m3), w.chrom_names))
    out["one_rec_total"] = np.asarray(loc1["rec_errors_total"], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, "rec trajectory", out["fit_rec_total"])


if __name__ == "__main__":
    only = set(sys.argv[1:])
    if only:
        if "rwr_conv" in only:
            make_rwr_conv_tiles()
        if "als_conv" in only:
            make_als("als_conv_small.npz", "small", 25, 40, 4, seed=3, do_conv=True)
        if "rwr_col" in only:
            make_rwr_col_tiles()
        if "als_col" in only:
            make_als("als_col_small.npz", "small", 25, 40, 4, seed=3, do_col=True)
        if "pack" in only:
            make_pack()
        if "postprocess" in only:
            make_postprocess()
        if "impute" in only:
            make_impute()
        if "multires" in only:
            make_multires()
        if "als_defaults" in only:
            make_als("als_defaults_small.npz", "small", 25, 40, 4, seed=3, do_conv=True,
                     do_rwr=False)
        if "als_bad" in only:
            make_als("als_bad_small.npz", "small", 25, 40, 4, seed=3, good_qc_num=80)
            make_als("als_badcol_small.npz", "small", 25, 40, 4, seed=3, do_col=True,
                     good_qc_num=80)
        sys.exit(0)
    make_rwr_tiles()
    make_rwr_conv_tiles()
    make_parafac()
    make_als("als_small.npz", "small", 25, 40, 4, seed=3)
    make_als("c1_fit.npz", "c1", None, None, 10, seed=1, save_U=False)
    make_als("als_conv_small.npz", "small", 25, 40, 4, seed=3, do_conv=True)
    make_rwr_col_tiles()
    make_als("als_col_small.npz", "small", 25, 40, 4, seed=3, do_col=True)
    make_als("als_bad_small.npz", "small", 25, 40, 4, seed=3, good_qc_num=80)
    make_als("als_badcol_small.npz", "small", 25, 40, 4, seed=3, do_col=True, good_qc_num=80)
    make_als("als_defaults_small.npz", "small", 25, 40, 4, seed=3, do_conv=True, do_rwr=False)
    make_pack()
    make_postprocess()
    make_impute()
    make_multires()
