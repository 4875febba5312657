"""Multi-process tests of bench.py's replica plumbing on CPU (gloo, world size 2): a single
LP does not shard, so N GPUs run N independent replicas joined only by a barrier and the
max / sum of their numbers; the reference arm runs on rank 0 alone."""
import json
import multiprocessing
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, port, queue):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    world, r, local, pg = bench.dist_setup(2)
    bench.barrier(pg)
    mx = bench.max_over_ranks(pg, float(rank + 1))
    sm = bench.sum_over_ranks(pg, 10.0 * (rank + 1))
    bench.barrier(pg)
    pg.destroy_process_group()
    queue.put((r, world, mx, sm))


def test_replicas_reduce_over_gloo():
    ctx = multiprocessing.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(queue.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.0, 30.0), (1, 2, 2.0, 30.0)]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--workload", "plain", "--cpu-sample-iters", "20"]
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
