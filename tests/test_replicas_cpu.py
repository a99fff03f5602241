"""The multi-GPU path of bench.py is replicas only: every rank runs its own
copy of the workload and the job's time is the slowest rank's.  The host
logic (max over ranks, whole-job rate) runs here on two gloo ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = 10.0 + 5.0 * rank  # rank 1 is the slow one
    ms = bench.max_over_ranks_of(ms_local, dist, "cpu")
    out.put((rank, ms, bench.job_rate(1000, 20, world, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(1000 * 20 * 2 / 0.015)


def test_captured_traffic_is_used_only_for_the_captured_source(tmp_path):
    """bench.py's roofline.traffic: the committed ncu figure of the step
    kernel counts only while the kernel's source has the SHA-256 stored with
    it."""
    import hashlib
    import json

    sys.path.insert(0, ROOT)
    import bench

    (tmp_path / "profiles").mkdir()
    (tmp_path / "fall3d_gb300" / "csrc").mkdir(parents=True)
    k = tmp_path / "fall3d_gb300" / "csrc" / "f3d_fused2.cu"
    assert bench.captured_traffic("step_fused", "cfg1", str(tmp_path)) == (None, "no capture")
    k.write_text("// kernel v1\n")
    sha = hashlib.sha256(k.read_bytes()).hexdigest()
    (tmp_path / "profiles" / "ncu_traffic.json").write_text(
        json.dumps({"cfg1": {"step_fused": 123456789, "kernel_sha256": sha}}))
    t, note = bench.captured_traffic("step_fused", "cfg1", str(tmp_path))
    assert t == 123456789 and "this kernel source" in note
    k.write_text("// kernel v2\n")
    t, note = bench.captured_traffic("step_fused", "cfg1", str(tmp_path))
    assert t is None and note.startswith("stale")
