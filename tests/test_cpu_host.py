"""CPU-only checks of the host side: the C ABI library, the Sparse container, the tiling."""
import os
import re

import numpy as np
import pytest

from fh_gb300 import _lib, synth
from fh_gb300.sparse_for_schic import Sparse, Chrom_Dataset, compact_layout
from oracle import fh_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "fhgb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fh_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_lib.LIB_PATH):
        from fh_gb300 import build
        build.build()
    lib = _lib.load()
    declared = header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    # the Python binding covers exactly the declared ABI
    assert sorted(_lib.SIGNATURES) == declared
    assert lib.fh_version() >= 100
    assert lib.fh_status_string(0) == b"ok"


def test_sparse_known_answers():
    """The reference's own known-answer test of Sparse (sparse_for_schic.py:634-661)."""
    def new_obj():
        return Sparse([[0, 2, 1, 0], [0, 3, 2, 1]], [1, 2, 3, 4.], (3, 4))
    base = new_obj().to_scipy().todense()
    o = new_obj(); o.sort_indices()
    assert (o.to_scipy().todense() == base).all()
    assert (new_obj().permute(0, 1).to_scipy().todense() == base).all()
    assert (new_obj().permute(1, 0).to_scipy().todense() == base.T).all()
    assert (new_obj().reshape(1, 12).to_scipy().todense() == base.reshape(1, 12)).all()
    assert (new_obj().reshape(4, 3).to_scipy().todense() == base.reshape(4, 3)).all()
    for s in [slice(2), slice(10), slice(0, None), slice(2, None), slice(1, 3)]:
        assert (new_obj().slicing(s).to_scipy().todense() == base[s]).all()
    o = new_obj().permute(1, 0).reshape(6, 2).slicing(slice(1, 3)).permute(1, 0)
    assert (o.to_scipy().todense() == base.T.reshape(6, 2)[1:3].T).all()


@pytest.mark.parametrize("num_bin,bs_bin,flank", [(37, 12, 4), (20, 12, 4), (249, 125, 20),
                                                  (5, 5, 10), (100, 100, 10), (130, 33, 30)])
def test_compact_layout_matches_oracle(num_bin, bs_bin, flank):
    mine = compact_layout(num_bin, bs_bin, flank)
    ref = O.tile_layout(num_bin, bs_bin, flank)
    assert len(mine) == len(ref)
    for a, b in zip(mine, ref):
        assert (a.start, a.rows, a.local, a.col, a.width, a.shift) == \
               (b.start, b.rows, b.local, b.col, b.width, b.shift)


def test_chrom_dataset_slices():
    w = synth.workload("tiny")
    coo, _ = synth.generate(w, seed=3)
    idx, val, shape = coo[0]
    d = Chrom_Dataset(Sparse(idx, val, shape), 12, 10, compact=True, flank=w.band)
    assert d.num_bin_batch == 4 and d.num_cell_batch == 3
    assert d.cell_slice_list == [slice(0, 10), slice(10, 20), slice(20, 24)]
    assert d.bin_slice_list[-1] == slice(36, 37)


def test_synthetic_generator_is_seeded():
    w = synth.workload("tiny")
    a, _ = synth.generate(w, seed=5)
    b, _ = synth.generate(w, seed=5)
    for (i1, v1, s1), (i2, v2, s2) in zip(a, b):
        assert s1 == s2 and (i1 == i2).all() and (v1 == v2).all()
    i, v, s = a[0]
    assert (np.abs(i[0] - i[1]) <= w.band).all()
    key = (i[0].astype(np.int64) * s[1] + i[1]) * s[2] + i[2]
    assert (np.diff(key) > 0).all()          # sorted by (row, col, cell), unique


def test_autotuner_picks_fastest_and_caches(tmp_path):
    from fh_gb300.autotune import Tuner
    cost = {4: 3.0, 2: 1.0, 8: 2.0}
    calls = []

    def timer(fn, reps):
        fn()
        return cost[calls[-1]]

    def run(c):
        calls.append(c)

    path = str(tmp_path / "tune.json")
    t = Tuner(path=path, enabled=True, timer=timer)
    assert t.choose("dev", "xg_splits", (10, 20), [4, 2, 8, 2], run) == 2
    assert sorted(set(calls)) == [2, 4, 8]
    n = len(calls)
    assert t.choose("dev", "xg_splits", (10, 20), [4, 2, 8], run) == 2   # memory cache
    assert len(calls) == n
    t2 = Tuner(path=path, enabled=True, timer=timer)                     # file cache
    assert t2.choose("dev", "xg_splits", (10, 20), [4, 2, 8], run) == 2
    assert len(calls) == n
    # ties keep the earlier candidate (the heuristic is listed first)
    cost.update({4: 1.0})
    assert Tuner(path="", enabled=True, timer=timer).choose("dev", "k", (1,), [4, 2], run) == 4


def test_autotuner_disabled_keeps_heuristic():
    from fh_gb300.autotune import Tuner

    def run(c):
        raise AssertionError("no timing when tuning is off")

    t = Tuner(path="", enabled=False, timer=lambda fn, reps: fn())
    assert t.choose("dev", "xg_splits", (1,), [7, 3, 14], run) == 7


class _FakeDeltas:
    """Stands in for FitEngine.auto_deltas: planted ||Q_e - Q_{e+1}||_F per (tile, cell)."""

    def __init__(self, deltas, n_good):
        self.d, self.C, self.Ct = deltas, n_good, deltas.shape[1]
        self.n_tiles = deltas.shape[0]
        self.tile_base = [0, 2]

    def auto_deltas(self, cap, all_cells=False):
        import torch
        out = torch.from_numpy(np.ascontiguousarray(self.d[:, :, :cap]))
        return out if all_cells else out[:, :self.C]


def test_auto_epochs_per_cell_batch():
    """partial_rwr.py:99-126 per cell batch: a batch stops at the first epoch whose largest
    delta over its cells is below 0.01 and keeps Q_{e+1}; 60 epochs without stopping keep Q_60;
    n_i is the largest stopping epoch over the good batches only (parafac2_intergrative.py:265)."""
    pytest.importorskip("torch")
    from fh_gb300.init import auto_epochs

    class D:   # two datasets of 2 bin batches, cells [0, 4) good in batches of 2, [4, 6) bad
        def __init__(self):
            self.num_bin_batch = 2
            self.num_cell_batch = 2
            self.cell_slice_list = [slice(0, 2), slice(2, 4), slice(4, 6)]

    rng = np.random.default_rng(0)
    d = rng.uniform(0.02, 1.0, size=(4, 6, 60)).astype(np.float32)
    stops = {(0, 0): 3, (0, 1): 5, (0, 2): 20, (1, 0): 0, (1, 1): None, (1, 2): 2,
             (2, 0): 14, (2, 1): 7, (2, 2): 1, (3, 0): 59, (3, 1): 4, (3, 2): None}
    for (t, b), e in stops.items():
        cs = D().cell_slice_list[b]
        if e is not None:
            d[t, cs, e] = 0.005          # every cell of the batch below 0.01 at epoch e
    eng = _FakeDeltas(d, 4)
    schic = [D(), D()]
    n_i, feat, cell_ep = auto_epochs(eng, schic, per_cell=True)
    want = np.zeros((4, 6), dtype=np.int32)
    for (t, b), e in stops.items():
        want[t, D().cell_slice_list[b]] = 60 if e is None else e + 1
    np.testing.assert_array_equal(cell_ep, want)
    stop = lambda t, b: 60 if stops[(t, b)] is None else stops[(t, b)]
    assert list(n_i) == [max(stop(t, b) for t in (0, 1) for b in (0, 1)),
                         max(stop(t, b) for t in (2, 3) for b in (0, 1))]
    np.testing.assert_array_equal(feat, [max(want[t, :4]) for t in range(4)])
    n_i2, feat2 = auto_epochs(eng, schic)       # the good batches alone give the same n_i
    np.testing.assert_array_equal(n_i2, n_i)
    np.testing.assert_array_equal(feat2, feat)


def _header_prototypes():
    """name -> list of parameter type strings, from the declarations in include/fhgb300.h."""
    txt = open(os.path.join(ROOT, "include", "fhgb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(fh_\w+)\s*\(([^;{]*?)\)\s*;", txt):
        params = " ".join(m.group(2).split())
        out[m.group(1)] = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
    return out


def test_ctypes_signatures_match_the_header():
    """Every ctypes binding has the header's parameter count, and each parameter's kind
    (pointer, 32-bit or 64-bit integer, size_t, float) matches its declared C type."""
    import ctypes as C
    protos = _header_prototypes()
    assert sorted(protos) == sorted(_lib.SIGNATURES)

    def kind(ctype):
        t = ctype.replace("const ", "").strip()
        if "*" in t:
            return C.c_void_p
        t = t.rsplit(" ", 1)[0] if " " in t else t
        return {"int32_t": C.c_int32, "int": C.c_int, "int64_t": C.c_int64, "size_t": C.c_size_t,
                "float": C.c_float, "double": C.c_double}[t]

    for name, (res, args) in _lib.SIGNATURES.items():
        params = protos[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for i, (a, p) in enumerate(zip(args, params)):
            want = kind(p)
            same = a is want or (C.sizeof(a) == C.sizeof(want) and
                                 a not in (C.c_float, C.c_double) and
                                 want not in (C.c_float, C.c_double) and
                                 (a is C.c_void_p) == (want is C.c_void_p))
            assert same, (name, i, p, a)


def test_bench_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (the reference's own fit on host cores, from its install under
    baseline/_ref) prints one JSON line with the keys the benchmark contract names, on the
    smallest workload; without the install it prints its unavailable line."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--config", "c1", "--steps", "1", "--warmup", "1", "--sample-cells", "40"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    if not os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "fasthigashi")):
        assert "unavailable" in line
        return
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["extrapolated"] is True
    assert cb["sample_cells"] == 40 and len(cb["measured_s"]) == 1
    # ms_per_step is the measured step, so steps x ms_per_step is the timed region
    assert abs(line["ms_per_step"] - 1000 * cb["measured_s"][0]) < 1.0
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_c_abi_rejects_bad_arguments_before_any_launch():
    """The entry points check their arguments before touching a device, and say why:
    FH_ERR_ARG (1) for malformed calls, FH_ERR_UNSUPPORTED for sizes past the kernels' range.
    Non-null dummy addresses are never dereferenced on these paths."""
    import ctypes as C
    if not os.path.exists(_lib.LIB_PATH):
        from fh_gb300 import build
        build.build()
    lib = _lib.load()
    p = C.c_void_p(16)                    # a dummy device address
    # malformed: null pointers, empty sizes, inconsistent shapes
    assert lib.fh_rwr_dense_f32(None, 4, 8, 12, 2, 3, p, None, None) == 1
    assert lib.fh_rwr_dense_f32(p, 4, 8, 12, 6, 3, p, None, None) == 1          # s0 + rows > width
    assert lib.fh_conv_dense_f32(p, 0, 8, 12, p, None) == 1
    assert lib.fh_polar_f32(p, 2, 8, 16, p, None, None, None) == 1              # n < r
    assert lib.fh_xe_f32(p, 100, 10, 100, p, 64, p, None) == 1                  # ldx % 128
    assert lib.fh_xe_f32(p, 128, 10, 100, p, 48, p, None) == 1                  # rp not 16/32/64/128
    assert lib.fh_cp_als(1, 1, p, p, p, p, p, 64, 64, 64, 64, -1, p, None, p, 1 << 20,
                         None, None) == 1                                       # n_iter < 0
    assert lib.fh_meta_polar(p, 100, 65, 64, p, p, p, 1 << 20, None, None) == 1  # R > rp
    assert lib.fh_rwr_col_dense(p, 4, 8, 12, 2, 3, None, p, None, None) == 1     # no coverage
    assert lib.fh_rwr_col_tiles(p, 1, 4, 8, 12, None, None, None, None, 12, None, p, None,
                                100, 0, None, None, None, None) == 1           # no segments
    # past the kernels' range
    unsup = lib.fh_polar_f32(p, 2, 300, 200, p, None, None, None)               # r > 128
    assert unsup not in (0, 1)
    assert lib.fh_status_string(unsup).decode() == lib.fh_status_string(
        lib.fh_meta_polar(p, 1000, 200, 256, p, p, p, 1 << 30, None, None)).decode()
    assert lib.fh_conv_dense_f32(p, 4, 200, 12, p, None) == unsup               # rows > 128


def test_product_path_raises_without_cuda():
    """No CPU fallback: the drop-ins refuse host tensors and the engine refuses a CPU device."""
    torch = pytest.importorskip("torch")
    from fh_gb300 import partial_rwr
    from fh_gb300.engine import FitEngine
    with pytest.raises(_lib.FHError):
        partial_rwr(torch.rand(2, 5, 9), 2, 7, False, True, False)
    with pytest.raises(_lib.FHError):
        FitEngine([], 4, {}, None, "cpu")


def test_parafac_sweep_schedule():
    """CP-ALS sweeps per fit iteration (parafac2_intergrative.py:636-637): one more every 10
    iterations after the first ten, capped at 10; the oracle's fit loop follows the same rule."""
    from fh_gb300.engine import FitEngine
    s = FitEngine.parafac_schedule(35, 1)
    assert s[:10] == [1] * 10 and s[10:20] == [2] * 10 and s[20:30] == [3] * 10 and s[30:] == [4] * 5
    assert FitEngine.parafac_schedule(200, 5)[-1] == 10
    assert FitEngine.parafac_schedule(3, 12) == [12, 12, 12]     # above the cap: left alone


def test_device_generator_gives_a_sorted_in_band_coo():
    """synth.generate_on_device (the 50,000-cell workload's generator), run here with torch on
    the CPU: every chromosome's COO is sorted by (row, column, cell) without repeats, inside the
    band and the shape, symmetric in (row, column), with positive values clipped at mean + 15 std;
    seeded; and close to the host generator's contact count."""
    import dataclasses
    from fh_gb300 import synth
    w = dataclasses.replace(synth.workload("tiny"), n_cells=40)
    coo, _ = synth.generate_on_device(w, seed=4, device="cpu", cell_chunk=16, band_chunk=7)
    again, _ = synth.generate_on_device(w, seed=4, device="cpu", cell_chunk=16, band_chunk=7)
    host, _ = synth.generate(w, seed=4)
    for (idx, val, shape), (idx2, val2, _), (hidx, _, _), nb in zip(coo, again, host, w.chrom_bins):
        assert shape == (nb, nb, w.n_cells) and idx.dtype == np.int32 and val.dtype == np.float32
        np.testing.assert_array_equal(idx, idx2)
        np.testing.assert_array_equal(val, val2)
        key = (idx[0].astype(np.int64) * nb + idx[1]) * w.n_cells + idx[2]
        assert (np.diff(key) > 0).all()
        assert (idx >= 0).all() and (idx[0] < nb).all() and (idx[1] < nb).all()
        assert (idx[2] < w.n_cells).all() and (np.abs(idx[0] - idx[1]) <= w.band).all()
        mirror = np.sort((idx[1].astype(np.int64) * nb + idx[0]) * w.n_cells + idx[2])
        np.testing.assert_array_equal(np.sort(key), mirror)
        assert (val > 0).all()
        assert abs(idx.shape[1] - hidx.shape[1]) < 0.1 * hidx.shape[1]
