"""Host logic of bench.py on the CPU: the byte model, the replicas-only
multi-process timing (world size 2 over gloo), the reference arm's
rank-0-only output and the CPU baseline's sampling."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_pair_bytes_match_the_three_pass_model():
    # 8N + 80H bytes per 512^3 float32 r2c+c2r pair (6,463,422,464 B)
    nb = bench.algorithmic_bytes((512, 512, 512), 4)
    pair = sum(nb[k] for k in ("z_r2c", "y", "x", "x_inv", "y_inv", "z_c2r"))
    N, H = 512 ** 3, 512 * 512 * 257
    assert pair == 8 * N + 80 * H == 6_463_422_464


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank                     # rank 1 is the slower replica
    worst = bench.max_over_ranks(ms, world)
    value = bench.replicas_value(100, world, worst)
    with open(os.path.join(out, f"r{rank}.json"), "w") as f:
        json.dump({"max_ms": worst, "value": value}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_timing_over_gloo(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for g in got:
        assert g["max_ms"] == pytest.approx(15.0)
        # 2 ranks x 100 pairs in the slowest rank's 15 ms
        assert g["value"] == pytest.approx(2 * 100 / 0.015)


def test_reference_arm_prints_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    bench.main()
    assert capsys.readouterr().out == ""


def test_cpu_baseline_sample_is_chosen_once_and_repeats_whole_pairs():
    """The CPU baseline (oracle, all host threads) picks its sample once per
    grid and budget; a budget above one pair's time repeats whole pairs."""
    bench._CPU_FRACTION.clear()
    bench._CPU_ARRAYS.clear()
    n = (16, 12, 10)
    v1, s1, th = bench.cpu_pairs_per_s(n, budget_s=0.05, nthreads=2)
    v2, s2, _ = bench.cpu_pairs_per_s(n, budget_s=0.05, nthreads=2)
    assert v1 > 0 and v2 > 0 and th == 2
    assert s1 == s2 and s1.endswith("double, 2 threads")
    reps = int(s1.split(" x ")[0])
    assert reps >= 1 and "1.0000 of one 16x12x10 pair" in s1
    assert len(bench._CPU_FRACTION) == 1 and len(bench._CPU_ARRAYS) == 1
    bench._CPU_FRACTION.clear()
    bench._CPU_ARRAYS.clear()
