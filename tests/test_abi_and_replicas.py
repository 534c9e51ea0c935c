"""C ABI surface and the replica aggregation of bench.py (no GPU).

* libsphdem.so loads without a GPU, reports its ABI version and exports every
  function declared in include/*.h; the ctypes mirrors of the ABI structs
  have the library's own sizes.
* bench.py --gpus N runs N independent replicas (the step does not shard);
  the job time is the max over ranks, checked here with two gloo ranks.
* bench.py --impl reference (the reference algorithm on the host cores) prints
  one JSON line with the bench contract's keys, on the small dam break.
"""
import ctypes as C
import os
import re
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from warp_sph_gpt_gb300 import build

    build.build_cuda()
    from warp_sph_gpt_gb300 import _lib

    return _lib.load()


def declared_functions():
    names = set()
    for header in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(sphdem_\w+)\s*\(", text, flags=re.M))
    return names


def test_library_loads_and_exports_every_declared_symbol(lib):
    from warp_sph_gpt_gb300 import _lib

    names = declared_functions()
    assert len(names) >= 30
    for name in sorted(names):
        assert hasattr(lib, name), f"{name} declared in include/*.h but not exported"
    assert set(_lib.EXPORTED) == names  # the binding covers exactly the declared surface
    assert lib.sphdem_abi_version() == _lib.ABI_VERSION
    _lib.check_layout(lib)  # raises on any size mismatch


def test_invalid_calls_return_status_without_a_gpu(lib):
    assert lib.sphdem_sph_onestep(None, None, 0, 1, None) == 2
    assert b"null context" in lib.sphdem_last_error()
    assert lib.sphdem_neighbour_digest(None, 3, 1.0, None, None, None) == 2
    # the learned jump and the device-judged rollout validate before touching the GPU
    assert lib.sphdem_jump(None, None, None, 0, 0, None) == 2
    assert lib.sphdem_rollout(None, None, None, 0, 1, 0.01, 0, None, None) == 2
    assert lib.sphdem_rollout_kernels(None, 0, 1, 0, 0) == -1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [12.0, 20.0][rank]
    ms_max = bench.reduce_max(ms, world)
    out[rank] = bench.job_throughput(1000, 10, world, ms_max)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_time_is_max_over_ranks_gloo():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    expected = world * 1000 * 10 / 20.0e-3  # the slower replica sets the time
    assert out[0] == pytest.approx(expected) and out[1] == pytest.approx(expected)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_max(7.5, 1) == 7.5
    assert bench.job_throughput(100, 4, 1, 2.0) == pytest.approx(200000.0)


def test_reference_arm_line_on_host():
    import json
    import subprocess

    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "small",
                          "--steps", "2", "--warmup", "3", "--cpu-budget-s", "2"],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] >= 3 and d["value"] > 0
    assert d["value"] == pytest.approx((d["config"]["fluid"] + d["config"]["dem"]) / (d["ms_per_step"] * 1e-3))
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["measured"]["steps_timed_in_full"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
