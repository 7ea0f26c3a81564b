"""X held partly in host memory (an engine with hbm_budget, fh_gb300/xstream.py) against the
same fit with X resident, on a 6-chromosome workload whose budget streams at least three
windows through the two staging slots.

* the walk: the resident part and every host window hold exactly the resident engine's X
  (the streamed chromosomes walked into a slot with their band rows re-based; each dataset's
  contacts copied in through many double-buffered COO chunks);
* init_params through the streamed X passes: the same auto-stop epochs, and features equal to
  fp32 rounding amplified by the sketch (1e-3);
* the fit (captured into a CUDA graph, with the window copies as memcpy nodes) and transform
  from the same state: X^T E is computed row range by row range with the same sums, X G^T
  adds the ranges' sums, so the embeddings agree to fp32 rounding (1e-5 after one fit, 1e-4
  after a second, replayed one)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

CUDA = "cuda"


def _datasets(w, seed=0):
    from fh_gb300 import synth
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    coo, _ = synth.generate(w, seed=seed)
    ds = []
    for (idx, val, shape), name, nb in zip(coo, w.chrom_names, w.chrom_bins):
        bsb, bsc = synth.recommend_batches(w, nb, w.n_cells)
        ds.append(Chrom_Dataset(Sparse(idx, val, shape), bsb, bsc, compact=True, flank=w.band,
                                chrom=name, resolution=w.resolution))
    return ds


def _workload():
    from fh_gb300 import synth
    return synth.Workload("stream6", 800, [60, 50, 45, 40, 35, 30], 1_000_000, 10, (0.9, 1.3),
                          8_000, 0.6, 3, 16, 5)


def _model(w, precision, budget=None):
    from fh_gb300 import Fast_Higashi_core
    m = Fast_Higashi_core(w.rank, w.band, [w.resolution], precision=precision,
                          hbm_budget=budget).to(CUDA)
    return m


def _budget_for_windows(w, ds, precision, min_windows=3):
    """The smallest budget (reserve 0) whose plan streams at least min_windows windows, found
    by lowering the budget until the plan has them."""
    from fh_gb300.engine import FitEngine
    m = _model(w, precision)
    m._sizes(ds, w.dim1, None)
    elem = 4
    e0 = FitEngine(ds, w.rank, m.chrom2size, None, CUDA, precision=precision)
    total = e0.rows * e0.Ct * elem + e0._buffer_bytes() + (64 << 20)
    del e0
    for frac in np.linspace(1.0, 0.3, 71):
        b = int(total * frac)
        try:
            e = FitEngine(ds, w.rank, m.chrom2size, None, CUDA, precision=precision, hbm_budget=b)
        except Exception:
            continue
        n = len(e.xs.plan.windows)
        del e
        if n >= min_windows:
            return b
    raise AssertionError("no budget streams %d windows" % min_windows)


def _host_array(buf, dtype, shape):
    n = int(np.prod(shape))
    raw = (ctypes.c_uint8 * (n * np.dtype(dtype).itemsize)).from_address(buf.ptr)
    return np.frombuffer(raw, dtype=dtype).reshape(shape).copy()


@pytest.mark.parametrize("precision", ["bf16x2", "fp32"])
def test_streamed_x_matches_resident_x(precision, monkeypatch):
    from fh_gb300.engine import FitEngine
    monkeypatch.setattr(FitEngine, "BUDGET_RESERVE", 0)
    # 1 MiB of COO chunk buffers: every dataset's build runs through many chunks
    monkeypatch.setattr(FitEngine, "BUDGET_CHUNK", 1 << 20)
    w = _workload()
    ds = _datasets(w)
    budget = _budget_for_windows(w, ds, precision)

    torch.manual_seed(0)
    mA = _model(w, precision)
    mA._sizes(ds, w.dim1, None)
    mA.init_params(ds, False, True, False, seed=0)
    torch.manual_seed(0)
    mB = _model(w, precision, budget)
    mB._sizes(ds, w.dim1, None)
    mB.init_params(ds, False, True, False, seed=0)
    eA, eB = mA.engine, mB.engine
    assert eB.xs is not None and len(eB.xs.plan.windows) >= 3
    np.testing.assert_array_equal(np.asarray(mA.n_i), np.asarray(mB.n_i))
    torch.cuda.synchronize()

    # the walk's X, resident part and host windows, bit for bit
    plan = eB.xs.plan
    if precision == "fp32":
        XA = eA.X.cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(eB.xs.res[:, :plan.split].cpu().numpy().view(np.uint32),
                                      XA[:, :plan.split])
        for wi, win in enumerate(plan.windows):
            h = _host_array(eB.xs.host[wi], np.uint32, (eB.Ct, win.ld))
            np.testing.assert_array_equal(h[:, :win.x1 - win.x0], XA[:, win.x0:win.x1])
            assert not h[:, win.x1 - win.x0:].any()
    else:
        XA = eA.X16.view(torch.int16).cpu().numpy()
        np.testing.assert_array_equal(eB.xs.res.view(torch.int16)[:, :, :plan.split].cpu().numpy(),
                                      XA[:, :, :plan.split])
        for wi, win in enumerate(plan.windows):
            h = _host_array(eB.xs.host[wi], np.int16, (eB.planes, eB.Ct, win.ld))
            np.testing.assert_array_equal(h[:, :, :win.x1 - win.x0], XA[:, :, win.x0:win.x1])
            assert not h[:, :, win.x1 - win.x0:].any()
    np.testing.assert_array_equal(eA.sumsq.cpu().numpy(), eB.sumsq.cpu().numpy())

    # init_params' features through the streamed passes: the sketch's products over a window
    # start their 64-row sums at another row than over resident X (fp32 rounding apart), which
    # the small singular gaps of the trailing components amplify (measured 1.1e-4 at bf16x2)
    EA, EB = mA.meta_embedding.cpu().double(), mB.meta_embedding.cpu().double()
    assert float((EA - EB).norm() / EA.norm()) < 1e-3

    # the fit and transform from one state.  The first fit runs eagerly, the second replays
    # the captured graph from where the first ended; X G^T sums range by range over streamed X
    # (and with the autotuner's split count over resident X), so the two engines drift apart
    # at fp32 rounding: within 1e-5 after one fit, 1e-4 after two (measured up to 1.05e-5)
    state = ([a.clone() for a in mA.A_list], {k: v.clone() for k, v in mA.B_dict.items()},
             {k: v.clone() for k, v in mA.D_dict.items()}, mA.meta_embedding.clone())
    for m in (mA, mB):
        m.A_list, m.B_dict, m.D_dict, m.meta_embedding = (
            [a.clone() for a in state[0]], {k: v.clone() for k, v in state[1].items()},
            {k: v.clone() for k, v in state[2].items()}, state[3].clone())
    for fit_no, tol in ((0, 1e-5), (1, 1e-4)):
        for m in (mA, mB):
            m.fit(ds, size_ratio=w.dim1, n_iter_max=w.n_iter, n_iter_parafac=1, do_conv=False,
                  do_rwr=True, do_col=False, tol=0, run_init=False, verbose=False)
        fA, fB = mA.meta_embedding.cpu().double(), mB.meta_embedding.cpu().double()
        assert float((fA - fB).norm() / fA.norm()) < tol, fit_no
        # the loss is a difference of large terms; the range-by-range sums show in it at 1.5e-6
        np.testing.assert_allclose(mB.rec_errors_total, mA.rec_errors_total, rtol=tol)
    tA = mA.transform(ds, False, True, False)[1][3].cpu().double()
    tB = mB.transform(ds, False, True, False)[1][3].cpu().double()
    assert float((tA - tB).norm() / tA.norm()) < 1e-4
    assert eB.xs.link_bytes > 0


def test_pin_memory_moves_the_coo_into_page_locked_buffers():
    """Chrom_Dataset.pin_memory: the same indices and values, now in library-allocated
    page-locked buffers (so the contact build copies them at the link's rate)."""
    from fh_gb300 import _lib
    w = _workload()
    ds = _datasets(w)
    d = ds[0]
    idx0, val0 = np.array(d.tensor.indices, copy=True), np.array(d.tensor.values, copy=True)
    assert d.pin_memory() is d
    t = d.tensor
    assert _lib.host_pinned(t.indices.ctypes.data, t.indices.nbytes)
    assert _lib.host_pinned(t.values.ctypes.data, t.values.nbytes)
    np.testing.assert_array_equal(t.indices, idx0)
    np.testing.assert_array_equal(t.values, val0)
    p0 = t.indices.ctypes.data
    d.pin_memory()                               # a second call keeps the same buffers
    assert d.tensor.indices.ctypes.data == p0


def test_budget_refuses_the_walks_that_need_x_resident():
    """do_conv and do_col run their walks from dense tiles of X's layout: with a budget the
    engine refuses them up front."""
    from fh_gb300 import _lib
    from fh_gb300.engine import FitEngine
    w = _workload()
    ds = _datasets(w)
    m = _model(w, "bf16x2")
    m._sizes(ds, w.dim1, None)
    for kw in (dict(do_conv=True), dict(do_col=True)):
        with pytest.raises(_lib.FHError):
            FitEngine(ds, w.rank, m.chrom2size, None, CUDA, precision="bf16x2", hbm_budget=1 << 40,
                      **kw)


def test_streamed_x_with_two_resolutions(monkeypatch):
    """Three chromosomes at 1 Mb and at 500 kb (res_list: a chromosome's datasets share B and
    D and stream in the same window): init and fit through the streamed passes agree with the
    resident engine's."""
    import dataclasses
    from fh_gb300 import Fast_Higashi_core, synth
    from fh_gb300.engine import FitEngine
    from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset
    monkeypatch.setattr(FitEngine, "BUDGET_RESERVE", 0)
    monkeypatch.setattr(FitEngine, "BUDGET_CHUNK", 1 << 20)
    w1 = synth.Workload("mr1", 800, [60, 50, 45], 1_000_000, 8, (0.9, 1.3), 6_000, 0.6, 3, 12, 4)
    w2 = dataclasses.replace(w1, name="mr2", chrom_bins=[120, 100, 90], resolution=500_000)
    ds = []
    for w, seed in ((w1, 1), (w2, 2)):
        coo, _ = synth.generate(w, seed=seed)
        for (idx, val, shape), name, nb in zip(coo, w.chrom_names, w.chrom_bins):
            bsb, bsc = synth.recommend_batches(w, nb, w.n_cells)
            ds.append(Chrom_Dataset(Sparse(idx, val, shape), bsb, bsc, compact=True,
                                    flank=w.band, chrom=name, resolution=w.resolution))
    res_list = [1_000_000, 500_000]

    def model(budget=None):
        m = Fast_Higashi_core(w1.rank, w1.band, res_list, precision="bf16x2",
                              hbm_budget=budget).to(CUDA)
        m._sizes(ds, w1.dim1, None)
        return m

    m0 = model()
    e0 = FitEngine(ds, w1.rank, m0.chrom2size, None, CUDA, precision="bf16x2")
    total = e0.rows * e0.Ct * 4 + e0._buffer_bytes() + (64 << 20)
    del e0
    budget = None
    for frac in np.linspace(1.0, 0.3, 71):
        b = int(total * frac)
        try:
            e = FitEngine(ds, w1.rank, m0.chrom2size, None, CUDA, precision="bf16x2",
                          hbm_budget=b)
        except Exception:
            continue
        n = len(e.xs.plan.windows)
        del e
        if n >= 1:
            budget = b
            break
    assert budget is not None
    torch.manual_seed(0)
    mA = model()
    mA.init_params(ds, False, True, False, seed=0)
    torch.manual_seed(0)
    mB = model(budget)
    mB.init_params(ds, False, True, False, seed=0)
    assert mB.engine.xs is not None and mB.engine.multi
    np.testing.assert_array_equal(np.asarray(mA.n_i), np.asarray(mB.n_i))
    state = ([a.clone() for a in mA.A_list], {k: v.clone() for k, v in mA.B_dict.items()},
             {k: v.clone() for k, v in mA.D_dict.items()}, mA.meta_embedding.clone())
    for m in (mA, mB):
        m.A_list, m.B_dict, m.D_dict, m.meta_embedding = (
            [a.clone() for a in state[0]], {k: v.clone() for k, v in state[1].items()},
            {k: v.clone() for k, v in state[2].items()}, state[3].clone())
        m.fit(ds, size_ratio=w1.dim1, n_iter_max=w1.n_iter, n_iter_parafac=1, do_conv=False,
              do_rwr=True, do_col=False, tol=0, run_init=False, verbose=False)
    fA, fB = mA.meta_embedding.cpu().double(), mB.meta_embedding.cpu().double()
    assert float((fA - fB).norm() / fA.norm()) < 1e-5
    np.testing.assert_allclose(mB.rec_errors_total, mA.rec_errors_total, rtol=1e-5)
