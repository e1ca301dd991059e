"""The replica run over two ranks on the gloo backend (CPU): the timing
collectives bench.py uses under torchrun (barrier, max over ranks, whole-job
throughput), and the reference arm's rule that only rank 0 works."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    from magicube_gb300.replicas import Replicas
    reps = Replicas("gloo")
    reps.barrier()
    seconds = 1.0 + rank  # rank 1 is the slowest
    value = reps.throughput(100.0, seconds)
    slowest = reps.max(seconds)
    reps.barrier()
    Path(out, f"r{rank}.json").write_text(json.dumps({"world": reps.world, "value": value, "max": slowest}))
    reps.close()


def test_replicas_two_gloo_ranks(tmp_path):
    world, port = 2, _free_port()
    mp.start_processes(_rank, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn")
    for r in range(world):
        res = json.loads((tmp_path / f"r{r}.json").read_text())
        assert res["world"] == 2
        assert res["max"] == 2.0                   # the slowest rank's time
        assert res["value"] == 100.0 * 2 / 2.0     # units of all ranks / that time


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun only rank 0 runs the reference arm; rank 1 exits 0 and
    prints nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0
    assert res.stdout.strip() == ""
