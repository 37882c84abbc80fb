"""The N > 1 host paths on CPU with world size 2 over gloo (127.0.0.1): the
bench's max-over-ranks timing, the instance sharding of the batched path
(every instance on exactly one rank, balanced by elements, the loss mean
recovered with one scalar reduction), and the reference arm launched by
torch.distributed.run (rank 0 prints the one JSON line, rank 1 exits 0)."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, counts, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from folax_gb300.batched import shard_instances
    ms = bench.max_over_ranks(1.5 + rank)  # the slowest rank's time
    parts = shard_instances(counts, world)
    mine = parts[rank]
    # per-instance "losses" of this rank's shard, reduced to the global mean
    losses = np.sqrt(np.asarray(counts, dtype=np.float64)[mine])
    t = torch.tensor([losses.sum(), float(len(mine))], dtype=torch.float64)
    dist.all_reduce(t)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine.tolist())
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "mean": float(t[0] / t[1]), "parts": gathered}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_time_shard_and_reduce(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    rng = np.random.default_rng(11)
    counts = (rng.integers(16, 129, size=200) ** 2).tolist()  # uneven quad meshes, n ~ U{16..128}
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, counts, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = json.load(open(tmp_path / "rank0.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    assert r0["ms"] == r1["ms"] == 2.5
    assert r0["parts"] == r1["parts"]
    allidx = sorted(r0["parts"][0] + r0["parts"][1])
    assert allidx == list(range(len(counts)))  # each instance on exactly one rank
    loads = [sum(counts[i] for i in p) for p in r0["parts"]]
    assert abs(loads[0] - loads[1]) <= max(counts)  # greedy balance bound
    assert r0["mean"] == pytest.approx(np.sqrt(counts).mean(), rel=1e-12)
    assert r0["mean"] == r1["mean"]


def test_shard_instances_single_rank_and_determinism():
    from folax_gb300.batched import shard_instances
    counts = [5, 9, 9, 1, 7]
    assert [p.tolist() for p in shard_instances(counts, 1)] == [[0, 1, 2, 3, 4]]
    a = shard_instances(counts, 3)
    b = shard_instances(counts, 3)
    assert [p.tolist() for p in a] == [p.tolist() for p in b] == [[1, 3], [2], [0, 4]]  # loads 10, 9, 12
    with pytest.raises(ValueError):
        shard_instances(counts, 0)


def test_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone runs the reference arm and prints one JSON line; the
    other rank exits 0 without work."""
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # the same metric, unit and workload as the GPU arm's line
    assert line["metric"].startswith("M elements/s") and line["unit"] == "M elements/s"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"]["workload"].startswith("hex8 linear-elastic fused loss+adjoint, 64^3")
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
