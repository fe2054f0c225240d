"""The bench's multi-rank host logic on CPU (gloo, world size 2).  The
reconstruction has no collective on its data path (every rank reconstructs
its own batch); what the ranks share is the timing: each rank's times reduce
to their maximum on every rank, and the reference arm under torchrun runs on
rank 0 alone while the other ranks exit 0 without output."""
import json
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(dist, *values[rank])
    finally:
        dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps(got))


def test_max_over_ranks_single_process():
    import bench

    assert bench.max_over_ranks(None, 1.25, 2.0) == (1.25, 2.0)


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp

    values = [(1.5, 7.0), (2.5, 3.0)]  # (device ms, end-to-end ms) per rank
    mp.start_processes(_rank_main, args=(2, _free_port(), values, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for rank in range(2):
        assert json.loads((tmp_path / f"rank{rank}.json").read_text()) == [2.5, 7.0]


def test_reference_arm_under_torchrun(orc):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "1", "--warmup", "0"]
    proc = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert proc.returncode == 0, proc.stderr[-3000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, proc.stdout[-3000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
