"""Host-side logic of bench.py: byte accounting, clock parsing, the JSON
contract of the CPU reference arm, and the multi-process max-over-ranks
timing with the gloo backend (world size 2, CPU only)."""
import json
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def test_step_bytes_model():
    counts = {"curve_fragment": 1000, "merged_fragment": 600, "span": 100}
    sb = bench.step_bytes(counts, npairs=800, V=300, C=100, P=10, W=64, H=64, S=32, affine=False)
    assert sb["sort"] == 1000 * 24
    assert sb["resolve"] == 800 * 20 + 600 * 16 + (2 * 32) * 8 + 64 * 64 * 4
    assert all(v > 0 for v in sb.values())
    assert bench.frame_alg_bytes(counts, 300, 100, 10, 64, 64, 32) > sb["resolve"]


def test_clock_sampler_parsing():
    cs = bench.ClockSampler(0)

    class P:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    class T:
        def join(self, timeout=None):
            pass

    cs.proc, cs.t = P(), T()
    cs.lines = ["0, 1965, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Active",
                "0, 2070, 2070, 950.0, 0x0, Not Active, Not Active, Not Active, Not Active",
                "garbage"]
    out = cs.stop()
    assert out["sm_mhz"] == (1965 + 2070) / 2 and out["sm_max_mhz"] == 2070
    assert out["reasons"] == ["sw_power_cap"]


def test_reference_arm_json(monkeypatch, capsys):
    monkeypatch.setattr(bench, "BAND_ROWS", 4)
    args = type("A", (), {"steps": 2, "warmup": 1, "gpus": 1})()
    bench.run_reference(args, rank=0, world=1)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "Mpix/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["higher_is_better"] is True
    # both arms describe the same workload with the same config object
    assert line["config"] == bench.workload_config()
    assert line["metric"] == bench.METRIC


def test_reference_arm_silent_on_other_ranks(capsys):
    args = type("A", (), {"steps": 1, "warmup": 0, "gpus": 2})()
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    m = bench.allreduce_max(10.0 + 5.0 * rank, world)
    out[rank] = m
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == 15.0
