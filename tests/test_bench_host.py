"""Host side of bench.py, without a GPU: the reference arm's JSON line (it runs the reference's CPU
NMF on the host cores) and the replica path for N > 1 (barrier and max over ranks on gloo, rank 0
alone printing)."""
import json
import os
import re
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--n", "256", "--m", "256", "--r", "16", "--steps", "1", "--warmup", "0"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(nproc, *args):
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(nproc),
            "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), *args]


def _json_lines(out):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", *SMALL], cwd=ROOT,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "iters/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["config"]["workload"] == "large_euclidean_256x256_r16"
    assert d["e2e"] == {"value": d["value"], "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]


def test_reference_arm_two_ranks_prints_once():
    # the launch the N = 2 scaling run uses (torchrun's own options would swallow --n / --m, so the
    # default 8192 x 8192 workload; the arm times one bounded step of its sample)
    r = subprocess.run(_torchrun(2, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"),
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def test_replicas_barrier_and_max_over_two_gloo_ranks(tmp_path):
    script = tmp_path / "replica.py"
    script.write_text(textwrap.dedent("""
        import os, sys
        sys.path.insert(0, %r)
        import bench
        rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
        d = bench.Dist(world)
        d.barrier()
        m = d.max(10.0 + rank)
        d.barrier()
        d.close()
        print("rank %%d world %%d max %%.1f" %% (rank, world, m), flush=True)
    """ % ROOT))
    r = subprocess.run(_torchrun(2, str(script)), cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    # the ranks share the launcher's stdout, so their lines may run together
    got = sorted(re.findall(r"rank \d world \d max [\d.]+", r.stdout))
    assert got == ["rank 0 world 2 max 11.0", "rank 1 world 2 max 11.0"]
