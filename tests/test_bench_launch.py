"""bench.py's own multi-rank launch: with --gpus N and no torchrun
environment it relaunches itself under torch.distributed.run with N ranks
(127.0.0.1 rendezvous), and rank 0 alone prints the JSON line.  Run here
with the CPU reference arm, which needs no GPU."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.timeout(600)
def test_gpus_2_launches_two_ranks_and_prints_one_line(oracle):
    env = {k: v for k, v in __import__("os").environ.items()
           if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "Mrays/s" and d["value"] > 0
