"""bench.py's multi-rank plumbing on the CPU: two gloo ranks on 127.0.0.1.

The GPU arm runs one independent replica per rank; what ranks share is the
barrier around the timed region and the maximum of the ranks' times.  Both
are checked here with world_size 2, and so is the reference arm's rule that
rank 0 alone works and prints the one JSON line.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_barrier_and_max_over_ranks(tmp_path):
    script = tmp_path / "rank.py"
    script.write_text(
        "import json, sys\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "import bench\n"
        "dist, ws, rank, local = bench._dist()\n"
        "bench._barrier(dist)\n"
        "v = bench._max_over_ranks(dist, 1.5 + rank)\n"
        "bench._barrier(dist)\n"
        "print(json.dumps({'rank': rank, 'ws': ws, 'local': local, 'v': v}))\n")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert all(o["ws"] == 2 and o["v"] == 2.5 for o in outs)


def test_reference_arm_two_ranks_one_line(oracle_built):
    port = _free_port()
    env = dict(os.environ, LG_REF_BUDGET_S="2", OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "3", "--warmup", "1", "--nx", "6",
                        "--regions", "3"],
                       capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
