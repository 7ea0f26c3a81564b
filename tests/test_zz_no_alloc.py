"""The scratch-free scan entry point against the workspace one, through the C ABI.

fh_exclusive_scan_noalloc serves callers that cannot allocate device memory themselves: it
takes only the input and output buffers and keeps its scratch in a fixed array inside the
library.  This file is collected last so that a run stopping at its first failure has
already run every other test; it also passes on its own in a fresh process.

Sizes: the scan works in blocks of 2,048 counts; the block totals are scanned in chunks of
1,024, so n > 2,097,152 runs the multi-chunk path, and n = 8,191 x 2,048 (the largest size the
library's scratch array holds) writes its last entry.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib

pytestmark = pytest.mark.gpu

MAX_N = 8191 * 2048


def scan_with_workspace(counts):
    n = counts.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device=counts.device)
    ws_bytes = _lib.value("fh_scan_workspace", n)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=counts.device)
    _lib.call("fh_exclusive_scan", _lib.ptr(counts), n, _lib.ptr(out), _lib.ptr(ws), ws_bytes,
              _lib.stream_ptr())
    return out


def scan_noalloc(counts):
    n = counts.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device=counts.device)
    _lib.call("fh_exclusive_scan_noalloc", _lib.ptr(counts), n, _lib.ptr(out), _lib.stream_ptr())
    return out


def check(counts):
    ref = scan_with_workspace(counts)
    got = scan_noalloc(counts)
    torch.cuda.synchronize()
    assert torch.equal(got, ref)           # integer work: bit-exact
    expect = np.concatenate([[0], np.cumsum(counts.cpu().numpy().astype(np.int64))])
    assert np.array_equal(got.cpu().numpy(), expect)


def test_noalloc_scan_matches_workspace_scan_twice():
    g = torch.Generator(device="cpu").manual_seed(7)
    for n in (2_000_003, 68_000):              # two calls in a row, the larger first
        check(torch.randint(0, 5000, (n,), generator=g, dtype=torch.int32).cuda())


def test_noalloc_scan_multi_chunk_and_largest_size():
    """Past 1,024 blocks (the block totals' multi-chunk scan) and at the largest size, where
    the last scratch entry is written; each call follows a larger one, so stale scratch from
    the call before would show."""
    g = torch.Generator(device="cpu").manual_seed(11)
    for n in (MAX_N, 2_097_153, 5_000_000 + 77):
        check(torch.randint(0, 200, (n,), generator=g, dtype=torch.int32).cuda())


def test_noalloc_scan_rejects_sizes_beyond_its_scratch():
    counts = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    st = _lib.load().fh_exclusive_scan_noalloc(_lib.ptr(counts), MAX_N + 1, _lib.ptr(out),
                                               _lib.stream_ptr())
    assert st == 2   # FH_ERR_UNSUPPORTED, before any launch
    assert int(out.sum().item()) == 0
