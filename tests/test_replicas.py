"""The N-GPU path of bench.py runs independent replicas (each rank its own tomograms,
no data-path collective): the job's time is the slowest rank's, its rate counts every
rank's tomograms, and only rank 0 prints.  Checked on CPU with gloo ranks."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    vals = bench.reduce_max([rank + 1.0, 10.0 - rank, 3.5], device="cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump(vals, f)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert json.load(open(tmp_path / f"r{r}.json")) == [2.0, 10.0, 3.5]


def test_max_without_a_process_group():
    import bench
    assert bench.reduce_max([1.5, 2]) == [1.5, 2.0]


def test_whole_job_rate_counts_every_rank():
    import bench
    # 4 replicas of 100 tomograms in 1000 ms (the slowest rank): 400 tomograms/s
    assert bench.whole_job_rate(4, 100, 1000.0) == pytest.approx(400.0)
    assert bench.whole_job_rate(1, 100, 500.0) == pytest.approx(200.0)


def _run_bench(args, rank, world):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(free_port()))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, env=env, capture_output=True,
                          text=True, timeout=120)


@pytest.mark.parametrize("args", [["--impl", "reference"], ["--config", "batched"], ["--config", "pocs"],
                                  ["--impl", "reference", "--config", "pocs"]])
def test_other_ranks_exit_without_output(args):
    """Rank 1 of 2: the reference arm and the one-GPU workloads print nothing and exit 0
    before touching a GPU (this container has none)."""
    r = _run_bench(args, 1, 2)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_rank_zero_reports_unavailable_workloads():
    r = _run_bench(["--impl", "reference", "--config", "pocs"], 0, 2)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line


def test_reference_arm_line_on_cpu():
    """The reference arm (the FP64 CPU restatement on the host cores) prints the bench
    line's contract: the metric, unit and direction of the GPU arm, a cpu_baseline that
    describes the run, and an e2e entry with no host-device copies."""
    r = _run_bench(["--impl", "reference", "--config", "plain_small", "--steps", "1", "--warmup", "3"], 0, 1)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "tomograms/s (hologram->RI)"
    assert line["unit"] == "tomograms/s" and line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"] == "plain_small"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "tomograms/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
