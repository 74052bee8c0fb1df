"""Host-side logic of bench.py, on CPU: the replica (N>1) aggregation over two gloo ranks, the
reference arm under torchrun-style ranks, and the roofline object's arithmetic."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_seconds = [0.5, 2.0][rank]  # rank 1 is the slow replica
    t = bench.max_over_ranks(local_seconds, dist, "cpu")
    dist.barrier()
    q.put((rank, t, bench.job_value(1000, 4, world, t)))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_gloo2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]
    # value = tests of all ranks / slowest time: 1000 tests x 4 steps x 2 ranks / 2 s
    assert [o[2] for o in out] == [4000.0, 4000.0]


def test_single_process_has_no_reduction():
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25


def _run_reference(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--workload", "sphere16k", "--steps", "1", "--warmup", "0",
                           "--cpu-seconds", "1"], capture_output=True, text=True, env=env,
                          timeout=600)


def test_reference_arm_rank0_prints_one_line():
    r = _run_reference({"RANK": "0", "WORLD_SIZE": "1"})
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["unit"] == "tests/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "tests/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _run_reference({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


class _Spec:
    ndiv2 = (8, 8, 8)


def test_roofline_fields():
    r = bench.roofline("torus262k", {"level2": 1.1, "level2_kernel": 1.0},
                       (10, 20, 30, 40), {"boundary": 100, "pairs": 1000}, _Spec(), 1000,
                       {"sm_max_mhz": 2000.0}, "measured", {})
    assert r["kernel"] == "k_level2c" and r["bound"] == "issue"
    assert r["peak"] == pytest.approx(4 * 152 * 2000e6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["achieved"] == pytest.approx(bench.LEVEL2_INST_PER_LAUNCH["torus262k"] / 1e-3 / 1e9)
    unknown = bench.roofline("nosuch", {"level2": 1.0}, (1, 1, 1, 1), {"boundary": 1, "pairs": 1},
                             _Spec(), 1, {"sm_max_mhz": 2000.0}, "measured", {})
    assert unknown["achieved"] is None and unknown["frac"] is None
