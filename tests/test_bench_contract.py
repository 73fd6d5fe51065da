"""The benchmark's reference arm runs on the host alone: one JSON line with the
metric, a positive value, the CPU baseline description and a zero-copy e2e."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "c0",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "Gvoxel/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["metric"].startswith("DAG-build Gvoxel/s")
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # the steps and warm-up given, and the GPU arm's config dict (bench.config_dict)
    assert d["steps"] == 1 and d["warmup"] == 1
    assert set(d["config"]) == {"workload", "map_side", "voxels_per_dag", "dag_words", "lookups_per_batch", "l2",
                                "parallelism"}
    assert d["config"]["map_side"] == 1024 and d["config"]["lookups_per_batch"] == 1 << 20


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the multi-GPU run is (torchrun, two ranks on one node,
    127.0.0.1 rendezvous), rank 0 alone runs and prints the line; the other
    rank exits 0 without work."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--config", "c0", "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def _replica_rank(rank, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        # rank 1 is the slower replica on the first time, rank 0 on the second
        ms = bench.slowest_rank(torch, [1.0 + rank, 4.0 - rank], 2, "cpu")
        q.put((rank, ms, bench.whole_job_rate(2, 1e9, ms[0])))
    finally:
        dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_over_gloo():
    """The N>1 form of the GPU arm: every replica builds its own workload, the
    job's time is the slowest rank's (an all-reduce of the times, the one
    collective), and the rate counts every replica's units."""
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in got:
        assert ms == [2.0, 4.0], (rank, ms)
        assert rate == 2 * 1e9 / 2e-3 / 1e9  # two replicas' units in the slowest 2 ms
