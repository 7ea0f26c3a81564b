"""The N > 1 host logic of bench.py on CPU: gloo process groups of world size 2."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=ROOT, env=env)


def test_reference_arm_two_ranks_prints_one_line():
    """Under torchrun with 2 ranks the reference arm runs on rank 0 alone, which prints the
    one JSON line (n_gpus = 2); the other rank exits 0 without work."""
    pytest.importorskip("torch")
    r = _torchrun(["bench.py", "--impl", "reference", "--config", "c1", "--gpus", "2",
                   "--steps", "1", "--warmup", "1", "--sample-cells", "40"])
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    if "unavailable" not in line:       # the reference is installed under baseline/_ref
        assert line["n_gpus"] == 2 and line["value"] > 0


def test_max_over_ranks_and_barrier(tmp_path):
    """Whole-job time is the slowest rank's: max_over_ranks on gloo, world size 2."""
    pytest.importorskip("torch")
    script = (
        "import sys, torch, torch.distributed as dist\n"
        "sys.path.insert(0, %r)\n"
        "import bench\n"
        "rank, local, ws = bench.dist_setup()\n"
        "assert ws == 2 and dist.get_backend() == 'gloo'\n"
        "dist.barrier()\n"
        "t = bench.max_over_ranks(torch.tensor([10.0 + 5.0 * rank]), ws)\n"
        "open(%r + '/rank%%d' %% rank, 'w').write('%%.1f' %% float(t.item()))\n"
        "dist.destroy_process_group()\n" % (ROOT, str(tmp_path)))
    path = tmp_path / "probe.py"
    path.write_text(script)
    r = _torchrun([str(path)], timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert [(tmp_path / ("rank%d" % k)).read_text() for k in (0, 1)] == ["15.0", "15.0"]
