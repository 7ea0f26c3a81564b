"""The bounded device-side waits, made to run out on purpose, without faulting the GPU.

Every mbarrier wait of the tensor-core kernels gives up after a time limit, sets FH_ERR_TIMEOUT
in the caller's status word and unwinds (tensor memory freed) instead of hanging the stream.
fh_selftest_wait takes that path with a wait nothing completes and a 1 ms limit: the call must
come back with the status set, the context must stay usable, and the next tensor-core pass
(which allocates tensor memory on the same SMs) must give the right answer.
"""
import math
import time

import pytest

torch = pytest.importorskip("torch")

from fh_gb300 import _lib

pytestmark = pytest.mark.gpu

CUDA = torch.device("cuda")
P = _lib.ptr


def test_wait_that_nothing_completes_times_out_and_the_next_call_runs():
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    t0 = time.perf_counter()
    _lib.call("fh_selftest_wait", P(st), 1_000_000, _lib.stream_ptr())
    torch.cuda.synchronize()
    took = time.perf_counter() - t0
    assert int(st.item()) == 7          # FH_ERR_TIMEOUT
    assert took < 5.0                   # the 1 ms limit, not a hang
    # two more in a row on the same stream: each times out and releases its tensor memory
    for _ in range(2):
        st.zero_()
        _lib.call("fh_selftest_wait", P(st), 200_000, _lib.stream_ptr())
        torch.cuda.synchronize()
        assert int(st.item()) == 7
    # the next tensor-core pass on the same device is unaffected
    C, rows, rp = 600, 1000, 64
    ldx = int(math.ceil(rows / 128) * 128)
    X = torch.zeros((C, ldx), device=CUDA)
    X[:, :rows] = torch.rand((C, rows), device=CUDA)
    X16 = X.to(torch.bfloat16).unsqueeze(0).contiguous()
    E = torch.randn((C, rp), device=CUDA)
    E2 = torch.empty((C, 2 * rp), dtype=torch.bfloat16, device=CUDA)
    _lib.call("fh_split_bf16", P(E), C, rp, rp, P(E2), _lib.stream_ptr())
    W = torch.full((rows, rp), float("nan"), device=CUDA)
    st.zero_()
    _lib.call("fh_xe_bf16", P(X16), ldx, C, 1, C, rows, P(E2), rp, 0, P(W), P(st),
              _lib.stream_ptr())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = X16[0, :, :rows].double().T @ (E2[:, :rp].double() + E2[:, rp:].double())
    assert float(torch.linalg.norm(W.double() - ref) / torch.linalg.norm(ref)) < 1e-5


def test_selftest_rejects_limits_outside_its_range():
    st = torch.zeros(1, dtype=torch.int32, device=CUDA)
    lib = _lib.load()
    assert lib.fh_selftest_wait(P(st), 0, _lib.stream_ptr()) == 1             # FH_ERR_ARG
    assert lib.fh_selftest_wait(P(st), 2_000_000_000, _lib.stream_ptr()) == 1
    assert lib.fh_selftest_wait(None, 1000, _lib.stream_ptr()) == 1
    torch.cuda.synchronize()
    assert int(st.item()) == 0
