"""bench.py's multi-process helpers on CPU: two gloo ranks over 127.0.0.1.

The engine's multi-GPU mode is replicas only (no collective on the data path); what
crosses ranks is the timing: a barrier around the timed region, the max of the ranks'
times and the sum of their tests.  The reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
d = bench.Dist()
d.barrier()
r = d.rank
out = {"rank": r, "world": d.world, "max": d.max(1.5 + r), "sum": d.sum(10 * (r + 1))}
d.barrier()
d.close()
print(json.dumps(out))
"""


def test_dist_helpers_two_gloo_ranks(tmp_path):
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), FPGM_DIST_BACKEND="gloo")
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["max"] == 2.5
        assert o["sum"] == 30


def test_reference_arm_prints_one_line_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--config", "c1", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["n_gpus"] == 2
    assert j["cpu_baseline"]["kind"] == "port" and j["value"] > 0
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0


def test_roofline_traffic_comes_from_the_committed_profiles():
    """bench.py's roofline `traffic` is read from the ncu summaries under profiles/: the DRAM
    bytes and algorithmic bytes of one captured launch, and which kernel was captured."""
    sys.path.insert(0, ROOT)
    import bench
    dram, alg, kernel = bench.profiled_traffic(("ci_part_kernel", "ci_compact_kernel"), "c4")
    assert kernel == "ci_part_kernel" and dram > 0 and alg > 0
    dram, alg, kernel = bench.profiled_traffic(("ci_warp_kernel",), "c2")
    assert kernel == "ci_warp_kernel" and 0 < dram < alg  # the c2 dataset stays in L2
    assert bench.profiled_traffic(("ci_warp_kernel",), "c3") is None


def test_counting_phase_fraction_sums_both_kernel_groups():
    """The counting-phase roofline figure is total algorithmic bytes over total event time of
    both kernel groups (e.g. 4 GB in 1 s and 1 GB in 4 s: 1 GB/s)."""
    sys.path.insert(0, ROOT)
    import bench
    r = bench.counting_phase([(1000.0, 4e9), (4000.0, 1e9)], 10.0)
    assert abs(r["achieved"] - 1.0) < 1e-12 and abs(r["frac"] - 0.1) < 1e-12 and r["kernel_ms"] == 5000.0
    assert bench.counting_phase([], 10.0) is None


_REF_ARM = r"""
import argparse, sys
sys.path.insert(0, sys.argv[1])
import bench
a = argparse.Namespace(gpus=1, steps=1, warmup=0, impl="reference", config="c1", alpha=0.05)
bench.run_reference(a, bench.Dist())
maps = open("/proc/self/maps").read()
print("ENGINE_LOADED" if "libfastpgm_gb300" in maps else "ENGINE_NOT_LOADED")
print("ORACLE_LOADED" if "liboracle" in maps else "ORACLE_NOT_LOADED")
"""


def test_reference_arm_never_loads_the_engine_library():
    """The reference arm times the reference algorithm's CPU port and generates its inputs
    with the oracle's copy of the seeded sampler: the engine's own library stays unloaded, and
    its config object is the one the GPU arm prints."""
    r = subprocess.run([sys.executable, "-c", _REF_ARM, ROOT], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ENGINE_NOT_LOADED" in r.stdout and "ORACLE_LOADED" in r.stdout, r.stdout
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    a = argparse.Namespace(gpus=1, config="c1", alpha=0.05)
    assert line["config"] == bench.bench_config(a, 1000)


def test_oracle_sampler_is_the_engine_sampler():
    """The oracle's separately built sampler gives the engine's bytes (both compile the same
    source with the same floating-point flags)."""
    import numpy as np
    import fastpgm_gb300 as F
    from oracle import oracle as O
    kw = dict(n_nodes=40, n_samples=3000, seed=9, avg_indegree=1.5, max_indegree=3, card=(2, 9), tail=(0.2, 10, 21),
              dirichlet=0.3)
    a, ca, pa = F.generate(**kw)
    b, cb, pb = O.generate(**kw)
    assert np.array_equal(a, b) and np.array_equal(ca, cb) and np.array_equal(pa, pb)
