"""The replica bookkeeping of bench.py on two gloo ranks on the host (no GPU): several GPUs run
independent operating points with no device exchange, and the host side only joins the ranks
(barrier), takes the slowest rank's time (max over ranks) and lets rank 0 alone print the line."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, tmp_path, timeout=900):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_max_over_ranks_and_barrier(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(
        "import json, os, sys\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "import bench\n"
        "rank, world, dist = bench.dist_init()\n"
        "bench.barrier(dist)\n"
        "t = bench.allmax(dist, 10.0 + rank)\n"
        f"open(os.path.join({str(tmp_path)!r}, 'rank%d.json' % rank), 'w').write("
        "json.dumps({'rank': rank, 'world': world, 'max': t}))\n"
        "dist.destroy_process_group()\n")
    r = _torchrun([str(script)], tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
    rows = [json.load(open(tmp_path / f"rank{q}.json")) for q in range(2)]
    assert sorted(x["rank"] for x in rows) == [0, 1]
    assert all(x["world"] == 2 and x["max"] == 11.0 for x in rows)


def test_reference_arm_prints_one_line_from_rank_zero(tmp_path):
    r = _torchrun([os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                   "--warmup", "3"], tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
