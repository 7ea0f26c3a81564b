"""The plan and the copy schedule of X held partly in host memory (fh_gb300/xstream.py), on
the CPU: which chromosomes stream, how they group into windows, the staging size, and the order
in which a pass reads the resident rows and the windows and copies windows into the two slots."""
import itertools

import numpy as np
import pytest

from fh_gb300 import _lib, synth, xstream


def chrom_rows_of(w):
    rows, x = [], 0
    for nb in w.chrom_bins:
        bsb, _ = synth.recommend_batches(w, nb, w.n_cells)
        t = 0
        for r0 in range(0, nb, bsb):
            r = min(bsb, nb - r0)
            t += r * (min(nb, r0 + r + w.band) - max(0, r0 - w.band))
        rows.append((x, x + t))
        x += t
    return rows


def nbytes(r, C, e):
    return -(-r // 128) * 128 * C * e


def test_everything_resident_when_it_fits():
    rows = [(0, 1000), (1000, 1700), (1700, 2000)]
    p = xstream.plan_x(rows, 4, 100, [800, 500, 300], 10 ** 9)
    assert p.windows == [] and p.split == 2000 and p.ld_res == 2048
    assert p.res_bytes == 2048 * 100 * 4
    assert p.staging_bytes >= 800 + (256 << 20)


def test_c5_shapes_stream_the_last_chromosomes_within_the_budget():
    """The 50,000-cell, R = 128 workload in two bf16 planes (179 GB) under a 173 GB X budget."""
    w = synth.workload("c5")
    rows = chrom_rows_of(w)
    ent = [int(8 * 7.0e9 * nb / sum(w.chrom_bins)) for nb in w.chrom_bins]
    budget = 173.4e9
    p = xstream.plan_x(rows, 4, w.n_cells, ent, budget)
    assert 0 < len(p.windows) <= 4
    assert p.res_bytes + p.staging_bytes <= budget
    assert p.split == p.windows[0].x0 and p.windows[-1].x1 == rows[-1][1]
    for a, b in zip(p.windows, p.windows[1:]):
        assert a.x1 == b.x0 and a.chroms[-1] + 1 == b.chroms[0]
    assert all(wd.nbytes <= p.slot_bytes for wd in p.windows)
    assert p.staging_bytes >= 2 * p.slot_bytes and p.staging_bytes >= max(ent) + (256 << 20)
    # streaming one chromosome fewer does not fit
    j = p.windows[0].chroms[0]
    assert nbytes(rows[j][1], w.n_cells, 4) > budget - 2 * p.slot_bytes or j == len(rows) - 1


def test_no_split_fits_raises():
    rows = [(0, 1000), (1000, 2000)]
    with pytest.raises(_lib.FHError):
        xstream.plan_x(rows, 4, 100, [0, 0], 1000)


def _brute_min_slot(rows, j, C, e, max_windows):
    """Smallest largest-window size over every split of chromosomes j.. into at most
    max_windows contiguous groups."""
    n = len(rows)
    m = n - j
    best = None
    for k in range(1, min(max_windows, m) + 1):
        for cuts in itertools.combinations(range(1, m), k - 1):
            bounds = [0, *cuts, m]
            big = max(nbytes(rows[j + bounds[i + 1] - 1][1] - rows[j + bounds[i]][0], C, e)
                      for i in range(k))
            best = big if best is None else min(best, big)
    return best


@pytest.mark.parametrize("seed", range(6))
def test_plan_streams_the_fewest_chromosomes_with_the_smallest_slots(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 9))
    sizes = rng.integers(200, 3000, n)
    rows, x = [], 0
    for s in sizes:
        rows.append((x, x + int(s)))
        x += int(s)
    C, e = 50, 4
    ent = [int(v) for v in rng.integers(0, 200_000, n)]
    total = nbytes(x, C, e)
    budget = int(total * rng.uniform(0.55, 0.9)) + (300 << 20)
    try:
        p = xstream.plan_x(rows, e, C, ent, budget, max_windows=3)
    except _lib.FHError:
        p = None

    def up(v):
        return -(-v // xstream.SLOT_ALIGN) * xstream.SLOT_ALIGN

    def staging(j, slot):
        ent_res = max([ent[c] for c in range(j)], default=0)
        ent_str = max([ent[c] for c in range(j, n)], default=0)
        slot = up(slot)
        chunk = 256 << 20
        v = max(2 * slot, up(ent_res) + chunk, (slot + up(ent_str) + chunk) if j < n else 0)
        return up(v)

    feasible = []
    for j in range(n, -1, -1):
        res = nbytes(rows[j][0], C, e) if j < n and rows[j][0] > 0 else (0 if j < n else total)
        slot = _brute_min_slot(rows, j, C, e, 3) if j < n else 0
        if res + staging(j, slot) <= budget:
            feasible.append((j, slot))
    if not feasible:
        assert p is None
        return
    j, slot = feasible[0]                       # the fewest chromosomes streamed
    assert p is not None
    assert (p.windows[0].chroms[0] if p.windows else n) == j
    assert max((wd.nbytes for wd in p.windows), default=0) == slot


class _FakeStream:
    def __init__(self, log):
        self.log = log

    def wait_event(self, ev):
        self.log.append(("wait", ev))


def _fake_xstream(n_windows, split=1):
    """An XStream with its copies and views replaced by records of what they would do."""
    xs = xstream.XStream.__new__(xstream.XStream)
    wins = [xstream.Window((i,), 10 * i + 10, 10 * i + 20, 128, 1000) for i in range(n_windows)]
    xs.plan = xstream.XPlan(10 * n_windows + 10, split, 128, 1, wins, 1024, 2048)
    xs.slot_win = [None, None]
    xs.res = "resident rows"
    content = [None, None]
    log = []

    def load(s, wi, main):
        content[s] = wi
        xs.slot_win[s] = wi
        log.append(("load", s, wi))
        return ("loaded", s, wi)

    xs._load = load
    xs.view = lambda s, wi: (s, wi)
    xs._main = lambda stream: stream
    return xs, content, log


@pytest.mark.parametrize("n_windows", [1, 2, 3, 4, 5])
def test_pass_order_reads_each_window_once_from_the_slot_that_holds_it(n_windows):
    xs, content, log = _fake_xstream(n_windows)
    main = _FakeStream(log)
    loads_per_pass = []
    for p in range(6):
        seen, res = [], []
        n0 = sum(1 for r in log if r[0] == "load")

        def win_fn(view, w):
            s, wi = view
            assert content[s] == wi                # the slot holds this window when it is read
            seen.append(wi)

        xs.run_pass(lambda X, rows: res.append(rows), win_fn, main)
        assert sorted(seen) == list(range(n_windows)) and res == [1]
        loads_per_pass.append(sum(1 for r in log if r[0] == "load") - n0)
    # after the first pass, only the windows beyond the two slots are copied in again
    assert all(v == max(0, n_windows - 2) for v in loads_per_pass[1:])
    assert loads_per_pass[0] == n_windows


def test_copies_of_later_windows_are_issued_before_the_resident_rows():
    """With four windows, the two copies a pass needs are issued before the resident rows are
    read (each as soon as the window read before it frees its slot), so they run behind that
    read on the copy stream."""
    xs, content, log = _fake_xstream(4)
    main = _FakeStream(log)
    xs.run_pass(lambda X, rows: None, lambda v, w: None, main)     # from empty slots
    for _ in range(3):
        log.clear()
        xs.run_pass(lambda X, rows: log.append(("res",)), lambda v, w: log.append(("win", v[1])),
                    main)
        kinds = [r[0] for r in log]
        loads = [i for i, k in enumerate(kinds) if k == "load"]
        assert len(loads) == 2 and kinds.index("res") > max(loads)
        # the windows read first are the two the previous pass ended with
        wins = [r[1] for r in log if r[0] == "win"]
        assert wins[:2] != wins[2:]


@pytest.mark.parametrize("nnz,buf,arrays", [(0, 1 << 20, 3), (1, 1 << 20, 4), (100_000, 1 << 20, 3),
                                            (12_345_677, 7 << 20, 4), (5_000, 3000, 3)])
def test_coo_chunks_cover_every_contact_once_inside_their_half(nnz, buf, arrays):
    """The budgeted contact build's chunking (sparse_for_schic.coo_chunks): chunks cover the
    contacts in order, each chunk's array slots lie inside its half of the buffer without
    overlapping, start on 256-byte boundaries, and consecutive chunks alternate halves."""
    from fh_gb300.sparse_for_schic import coo_chunks
    if nnz and (buf // 2) // 256 * 256 // (4 * arrays) < 64:
        with pytest.raises(_lib.FHError):
            coo_chunks(nnz, buf, arrays)
        return
    ch = coo_chunks(nnz, buf, arrays)
    half = (buf // 2) // 256 * 256
    nxt = 0
    for j, (b, offs, e0, m) in enumerate(ch):
        assert b == j % 2 and e0 == nxt and m > 0
        nxt += m
        assert len(offs) == arrays
        spans = sorted((o, o + 4 * m) for o in offs)
        for (a0, a1), (c0, _) in zip(spans, spans[1:]):
            assert a1 <= c0
        assert all(o % 256 == 0 for o in offs)
        assert spans[0][0] >= b * half and spans[-1][1] <= (b + 1) * half
        if j + 1 < len(ch):
            assert m % 64 == 0
    assert nxt == nnz


def test_staging_layout_keeps_windows_segments_and_chunks_apart():
    """XStream's views of the staging area (a CPU tensor stands in for the device one): each
    slot view of each window lies inside its slot; a resident dataset's segments and COO chunks
    start at the staging start, a streamed dataset's after slot 0 (which its walk writes), and
    segments and chunk room never overlap or leave the staging area."""
    import torch
    w = synth.workload("c5")
    rows = chrom_rows_of(w)
    ent = [int(8 * 7.0e9 * nb / sum(w.chrom_bins)) for nb in w.chrom_bins]
    for elem, planes, dtype in ((4, 2, torch.bfloat16), (4, 1, torch.float32)):
        p = xstream.plan_x(rows, elem, 500, [e // 100 for e in ent], 1.70e9)
        assert p.windows
        xs = xstream.XStream.__new__(xstream.XStream)
        xs.plan, xs.planes, xs.C, xs.dtype, xs.torch = p, planes, 500, dtype, torch
        xs.elem = torch.tensor([], dtype=dtype).element_size()
        xs.staging = torch.zeros(p.staging_bytes, dtype=torch.uint8)
        base = xs.staging.data_ptr()
        for wi, win in enumerate(p.windows):
            for s in (0, 1):
                v = xs.view(s, wi)
                assert v.shape == ((planes, 500, win.ld) if dtype == torch.bfloat16 else (500, win.ld))
                lo = v.data_ptr() - base
                assert lo == s * p.slot_bytes and lo + v.numel() * xs.elem <= (s + 1) * p.slot_bytes
        first = p.windows[0].chroms[0]
        ent_res = max(e // 100 for e in ent[:first])
        ent_str = max(e // 100 for e in ent[first:])
        for streamed, emax in ((False, ent_res), (True, ent_str)):
            for e in (0, 1 << 20, emax):           # what the plan sized the staging for
                seg, buf, nbuf = xs.build_space(streamed, e)
                start = p.slot_bytes if streamed else 0
                assert seg - base == start
                assert buf - base >= start + e and buf % (2 << 20) == base % (2 << 20)
                assert buf - base + nbuf == p.staging_bytes and nbuf >= 256 << 20
