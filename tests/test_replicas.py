"""The N > 1 form of bench.py on CPU: the path does not shard, so N GPUs run N independent
replicas; what the ranks share is the timing (barriers around the timed region, the slowest
rank's duration by an all-reduce MAX) and the whole-job value.  Two `gloo` ranks stand in for the
GPUs here; the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, times, out_dir: str):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        t = bench.max_over_ranks(times[rank], dist, device="cpu")
        dist.barrier()
        v = bench.replica_value(world, 10, t)
        Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"t": t, "v": v}))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_value_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    times = [120.0, 180.0]
    mp.start_processes(_rank_main, args=(2, _free_port(), times, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    for r in res:
        assert r["t"] == 180.0                       # every rank sees the slowest rank's duration
        assert r["v"] == pytest.approx(2 * 10 / 0.180)  # both replicas' steps over that duration


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replica_value(1, 20, 125.0) == pytest.approx(160.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank starts bench.py --impl reference; the ranks other than 0 exit 0
    at once without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
