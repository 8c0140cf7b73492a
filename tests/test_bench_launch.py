"""bench.py --gpus N without torchrun relaunches itself as N ranks (one
process per GPU) and each rank sees the torchrun environment; the N = 1 path
runs in-process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_rank_launch_command():
    sys.path.insert(0, ROOT)
    import bench
    cmd = bench.rank_launch_command(["--gpus", "4", "--steps", "3"], 4, port=29511)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "--master-addr=127.0.0.1" in cmd
    assert "--master-port=29511" in cmd
    assert cmd[-4:] == ["--gpus", "4", "--steps", "3"]


def test_gpus_2_spawns_two_ranks():
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2",
                        "--print-rank-env"], capture_output=True, text=True, timeout=300,
                       env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(rows) == 2, r.stdout
    assert sorted(int(x["RANK"]) for x in rows) == [0, 1]
    assert sorted(int(x["LOCAL_RANK"]) for x in rows) == [0, 1]
    assert all(x["WORLD_SIZE"] == "2" and x["MASTER_ADDR"] == "127.0.0.1" for x in rows)


def test_gpus_1_runs_in_process():
    env = {k: v for k, v in os.environ.items() if k != "WORLD_SIZE"}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--print-rank-env"],
                       capture_output=True, text=True, timeout=120, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(rows) == 1 and rows[0]["WORLD_SIZE"] is None
