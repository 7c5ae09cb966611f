"""Host-side logic of bench.py, on CPU: the max over replicas at world size 2 (gloo), the reference
arm's rank rule, and the Karger-Stein work model."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        # each replica's own time; the job's time is the slowest one's
        got = bench._max_over_ranks(3.0 + 4.0 * rank, 2)
        with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
            f.write(repr(got))
    finally:
        dist.destroy_process_group()


def test_max_over_two_replicas_on_gloo(tmp_path):
    mp.spawn(_replica, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    assert [float((tmp_path / ("r%d" % r)).read_text()) for r in range(2)] == [7.0, 7.0]


def test_single_process_needs_no_group():
    import bench
    assert bench._max_over_ranks(2.5, 1) == 2.5


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank but 0 exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                         capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == ""


def test_ks_work_model_matches_the_byte_model():
    """B(n) of one dense Karger-Stein trial: 6.8 MB at n = 318 and 3.64 GB at n = 4000 with 8-byte
    entries; 2048 leaves of 128 vertices under a K4000 root."""
    import bench
    assert bench._ks_work_model(318, 1.0, 8, 1.0, "x")["bytes_per_trial"] == 6769200
    k = bench._ks_work_model(4000, 1.0, 8, 1.0, "x")
    assert k["bytes_per_trial"] == 3638225936 and k["leaf_ops_per_trial"] == 2048 * 128 ** 3
    assert bench._ks_work_model(4000, 1.0, 4, 1.0, "x")["bytes_per_trial"] == 3638225936 // 2
