"""The N>1 path (replicas) with two gloo ranks on CPU: the camera shares cover every
camera exactly once, and whole-job throughput uses the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world_size, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "voxel-rt_gb300"))
    import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    mine = replicas.share(64, rank, world_size)
    gathered = [None] * world_size
    dist.all_gather_object(gathered, mine)
    t = replicas.max_over_ranks(1.0 + rank, dist)
    rate = replicas.whole_job_rate(len(mine), t, world_size)
    out[rank] = (gathered, t, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    world_size = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world_size, port, out), nprocs=world_size, join=True)
        res = dict(out)
    gathered, t0, rate0 = res[0]
    _, t1, rate1 = res[1]
    cams = sorted(c for part in gathered for c in part)
    assert cams == list(range(64))
    assert t0 == t1 == 2.0  # the slowest rank's time on every rank
    assert rate0 == rate1 == 64 / 2.0


def test_bench_reference_arm_under_torchrun_two_ranks(oracle):
    """bench.py --impl reference launched as the driver launches N > 1 (torchrun, two
    ranks): rank 0 alone times the CPU restatement and prints one JSON line, with the
    workload config of the GPU arm; the other rank exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(root, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.4"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["config"]["world"] == "512x256x512" and d["config"]["parallelism"] == "replicas x2"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_bench_reference_arm_under_two_ranks():
    """bench.py --impl reference launched as the N=2 run is launched (torchrun, one process
    per rank): rank 0 alone times the CPU restatement and prints the one JSON line, with
    n_gpus = 2 and the same config keys as the N=1 line; rank 1 exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
           os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.4"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=root)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(l) for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 1
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
    assert set(d["config"]) == {"workload", "world", "image", "max_steps", "local_lights", "seed", "l2",
                                "parallelism"}
    assert d["config"]["parallelism"] == "replicas x2"
