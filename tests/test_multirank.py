"""The N > 1 bench path (independent replicas, max time over ranks) and the
reference arm under several ranks, on CPU with the gloo backend."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 + 5.0 * rank, device="cpu")
    out[rank] = got
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == 15.0


def test_max_over_ranks_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.5, device="cpu") == 3.5


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_on_rank0_only(rank, tmp_path):
    env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0", "--cpu-sample", "20000"],
                       capture_output=True, text=True, env=env, cwd=REPO, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    if rank == 0:
        line = json.loads(lines[-1])
        assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
        assert line["e2e"]["h2d_bytes_per_step"] == 0
    else:
        assert lines == []


def test_clock_sampler_keeps_the_timed_region():
    """The clock record of a bench line: only the nvidia-smi samples that
    arrived inside the timed region count (the sampler starts before it),
    throttle reasons are read from those, and a region shorter than the
    sampling period takes the first sample after it."""
    sys.path.insert(0, REPO)
    import bench
    c = bench.ClockSampler(0)
    row = "0, {mhz}, 2070, 900.00, 0x0, Not Active, Not Active, Not Active, {cap}"
    c.lines = [(1.00, row.format(mhz=1200, cap="Not Active")),   # before: start-up
               (1.10, row.format(mhz=2070, cap="Not Active")),
               (1.20, row.format(mhz=2060, cap="Active")),
               (1.30, row.format(mhz=2070, cap="Not Active")),
               (1.45, row.format(mhz=900, cap="Not Active"))]    # after: idle
    c.window(1.05, 1.35)
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    c.window(1.31, 1.40)  # no sample inside: the first one after
    s = c.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 900.0 and s["reasons"] == []
    c.window(2.0, 2.1)  # nothing inside or after
    assert c.summary()["samples"] == 0
