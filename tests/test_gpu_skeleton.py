"""GPU PC-stable skeleton parity: batched engine and plain path against the reference's
golden sepsets/CPDAGs and the oracle's per-level deterministic test counts."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, read_sepsets, sepset_arrays
from oracle import oracle as O
import fastpgm_gb300 as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = F.Engine(0)
    yield e
    e.close()


def struct_of(tmp_path, names, res):
    edges = F.orient_cpdag(res["adj"], res["removed"], res["sep_offsets"], res["sep_vars"])
    p = str(tmp_path / "x_struct")
    F.write_struct(p, names, edges, int(res["adj"].sum()) // 2)
    return open(p).read()


@pytest.mark.parametrize("mode", [F.FPGM_MODE_BATCHED, F.FPGM_MODE_PLAIN])
def test_alarm_matches_reference_golden(eng, alarm, tmp_path, mode):
    names, cols, card = alarm
    eng.upload(cols, relabel=False)
    st = eng.pc_skeleton(mode=mode).to_dict()
    res = eng.result()
    assert res["sepsets"] == read_sepsets(os.path.join(GOLDEN, "alarm_sepsets"))
    assert st["tests"] == [666, 3579, 828, 118, 15]
    assert st["edges_after"] == [262, 67, 46, 44, 44]
    assert struct_of(tmp_path, names, res) == open(os.path.join(GOLDEN, "alarm_s5000_struct")).read()


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_synthetic_matches_reference(eng, tmp_path, name):
    raw, depth, _ = F.make_config(name)
    eng.upload(raw)
    st = eng.pc_skeleton(depth=depth).to_dict()
    res = eng.result()
    assert res["sepsets"] == read_sepsets(os.path.join(GOLDEN, name + "_sepsets"))
    n = raw.shape[0]
    assert struct_of(tmp_path, ["V%d" % i for i in range(n)], res) == open(os.path.join(GOLDEN, name + "_struct")).read()
    cols, card = O.relabel(raw)
    ref = O.pc_skeleton(cols, card, depth=depth, threads=16)
    assert st["tests"] == ref["stats"]["tests"]
    assert st["edges_after"] == ref["stats"]["edges_after"]
    assert all(e >= t for e, t in zip(st["tests_executed"], st["tests"]))


def test_plain_matches_batched_c1(eng):
    raw, depth, _ = F.make_config("c1")
    eng.upload(raw)
    sb = eng.pc_skeleton(mode=F.FPGM_MODE_BATCHED).to_dict()
    rb = eng.result()
    sp = eng.pc_skeleton(mode=F.FPGM_MODE_PLAIN).to_dict()
    rp = eng.result()
    assert rb["sepsets"] == rp["sepsets"] and np.array_equal(rb["adj"], rp["adj"])
    assert sb["tests"] == sp["tests"]


@pytest.mark.parametrize("name,S,nodes,depth", [("c3", 20000, None, 5), ("c4", 4000, 300, 1000),
                                                ("c4", 3000, None, 3)])
def test_other_shapes_match_oracle(eng, name, S, nodes, depth):
    raw, d0, _ = F.make_config(name, n_samples=S, n_nodes=nodes)
    cols, card = O.relabel(raw)
    eng.upload(raw)
    st = eng.pc_skeleton(depth=depth).to_dict()
    res = eng.result()
    ref = O.pc_skeleton(cols, card, depth=depth, threads=16)
    assert np.array_equal(res["adj"], ref["adj"])
    assert res["sepsets"] == ref["sepsets"]
    assert st["tests"] == ref["stats"]["tests"]


def test_depth_limits_levels(eng):
    raw, _, _ = F.make_config("c1")
    cols, card = O.relabel(raw)
    eng.upload(raw)
    for depth in (1, 2, 3):
        st = eng.pc_skeleton(depth=depth).to_dict()
        res = eng.result()
        ref = O.pc_skeleton(cols, card, depth=depth, threads=4)
        assert st["n_levels"] == ref["stats"]["n_levels"] == depth
        assert res["sepsets"] == ref["sepsets"]


def test_cli_and_python_binding_reproduce_alarm(alarm, tmp_path):
    names, cols, card = alarm
    csv = str(tmp_path / "alarm_s5000")
    with open(csv, "w") as f:
        f.write(",".join(names) + "\n")
        for s in range(cols.shape[1]):
            f.write(",".join(str(int(v)) for v in cols[:, s]) + "\n")
    out = subprocess.run([F.CLI_PATH, "-j", "0", "-m", "0", "-f2", csv], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    golden = open(os.path.join(GOLDEN, "alarm_s5000_struct")).read()
    assert open(csv + "_struct").read() == golden
    os.remove(csv + "_struct")
    # the reference driver's own import line, resolved through PYTHONPATH from another directory
    code = "import cmake_example as fastpgm; fastpgm.BNSL_PCStable(0, 1, 1, 0.05, '', %r, True)" % csv
    env = dict(os.environ, PYTHONPATH=ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=str(tmp_path), env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert open(csv + "_struct").read() == golden
    out = subprocess.run([F.CLI_PATH, "-j", "0", "-m", "0", "-e", "1", "-f2", csv], capture_output=True, text=True)
    assert out.returncode == 0
    assert open(csv + "_struct").read() == golden


def _small_jobs(n_jobs, seed, max_samples):
    jobs = F.c5_jobs(seed=seed, n_jobs=n_jobs)
    for j in jobs:  # the c5 generator with smaller datasets, so that the oracle stays quick
        j["n_nodes"] = min(j["n_nodes"], 60)
        j["n_samples"] = min(j["n_samples"], max_samples)
    return jobs


def test_several_datasets_match_each_oracle(eng):
    """Several independent datasets learned in one skeleton call (every level's tests of all
    datasets in the same waves) give each dataset's own skeleton, sepsets and test counts."""
    data, depth = F.make_jobs(_small_jobs(6, seed=55, max_samples=20000))
    eng.upload_jobs(data)
    st = eng.pc_skeleton(depth=depth).to_dict()
    res = eng.result()
    per_job = F.split_jobs(res, eng.job_offsets)
    levels = [0] * st["n_levels"]
    for raw, (adj, seps) in zip(data, per_job):
        cols, card = O.relabel(raw)
        ref = O.pc_skeleton(cols, card, depth=depth, threads=16)
        assert np.array_equal(adj, ref["adj"])
        assert seps == ref["sepsets"]
        assert ref["stats"]["n_levels"] <= st["n_levels"]
        for lv, t in enumerate(ref["stats"]["tests"]):
            levels[lv] += t
    assert st["tests"] == levels


def test_partitioned_strata_in_a_skeleton(monkeypatch, capfd):
    """A 70,000-sample dataset with 6-9 states per variable whose levels 5 and 6 test 8,000 to
    22,000 strata (beyond the shared hash: partitioned kernel), learned next to a small
    dataset in one skeleton call: each skeleton, sepset and test count equals the oracle's,
    and the wave log shows partitioned tests."""
    monkeypatch.setenv("FPGM_WAVE_LOG", "1")
    big, _, _ = F.generate(n_nodes=12, n_samples=70000, seed=72, n_edges=30, max_indegree=5, card=(6, 10))
    small, _, _ = F.generate(n_nodes=10, n_samples=5000, seed=73, n_edges=14, max_indegree=3, card=(2, 4))
    data = [big, small]
    with F.Engine(0) as e:
        e.upload_jobs(data)
        st = e.pc_skeleton().to_dict()
        res = e.result()
        offsets = e.job_offsets
    log = capfd.readouterr().err
    parts = [int(t) for t in re.findall(r"partitioned=(\d+)", log)]
    assert sum(parts) > 0, "no test reached the partitioned kernel"
    levels = [0] * st["n_levels"]
    for raw, (adj, seps) in zip(data, F.split_jobs(res, offsets)):
        cols, card = O.relabel(raw)
        ref = O.pc_skeleton(cols, card, threads=16)
        assert np.array_equal(adj, ref["adj"])
        assert seps == ref["sepsets"]
        for lv, t in enumerate(ref["stats"]["tests"]):
            levels[lv] += t
    assert st["tests"] == levels


def test_several_datasets_plain_matches_batched(eng):
    data, depth = F.make_jobs(_small_jobs(3, seed=56, max_samples=3000))
    eng.upload_jobs(data)
    sb = eng.pc_skeleton(depth=depth).to_dict()
    rb = eng.result()
    sp = eng.pc_skeleton(depth=depth, mode=F.FPGM_MODE_PLAIN).to_dict()
    rp = eng.result()
    assert np.array_equal(rb["adj"], rp["adj"]) and rb["sepsets"] == rp["sepsets"]
    assert sb["tests"] == sp["tests"]


def test_tests_across_datasets_are_rejected(eng):
    data, _ = F.make_jobs(_small_jobs(2, seed=57, max_samples=2000))
    eng.upload_jobs(data)
    n0 = data[0].shape[0]
    with pytest.raises(F.FpgmError, match="different datasets"):
        eng.ci_test(0, n0, ())
    with pytest.raises(F.FpgmError, match="mixes datasets"):
        eng.ci_test_batch(np.array([[0, 1, n0]], dtype=np.int32), 1)


def test_learning_job_reproduces_reference_files(tmp_path):
    """-j 1 -m 0 (BNL_PCStable): the learned CPDAG and the parameter file of the reference's own
    PC-stable + ParameterLearning run on c1 (tests/golden/c1_struct, c1_bnl_param), through
    the command line and through the Python binding."""
    raw, _, _ = F.make_config("c1")
    csv = str(tmp_path / "c1.csv")
    F.write_csv(csv, raw)
    out = subprocess.run([F.CLI_PATH, "-j", "1", "-m", "0", "-f2", csv, "-sp", "1"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert open(csv + "_struct").read() == open(os.path.join(GOLDEN, "c1_struct")).read()
    golden = open(os.path.join(GOLDEN, "c1_bnl_param")).read()
    assert open(csv + "_param").read() == golden
    os.remove(csv + "_param")
    from fastpgm_gb300 import cmake_example as fastpgm
    fastpgm.BNL_PCStable(0, 1, 1, 0.05, "", csv, True, True)
    assert open(csv + "_param").read() == golden


@pytest.mark.parametrize("alpha,depth,n,S", [(0.0, 1000, 12, 3000), (1.0, 1000, 12, 3000), (0.05, 0, 12, 3000),
                                             (0.05, 1, 12, 3000), (0.05, 1000, 2, 500), (0.05, 1000, 6, 1),
                                             (0.05, 1000, 9, 17)])
def test_edge_cases_match_oracle(eng, alpha, depth, n, S):
    """alpha 0 and 1, depth 0 and 1, two variables, one sample, a ragged 17 samples."""
    raw, _, _ = F.generate(n_nodes=n, n_samples=S, seed=21 + n + S, n_edges=max(1, n - 1),
                           max_indegree=min(3, n - 1), card=(2, 4))
    cols, card = O.relabel(raw)
    eng.upload(raw)
    st = eng.pc_skeleton(alpha=alpha, depth=depth).to_dict()
    res = eng.result()
    ref = O.pc_skeleton(cols, card, alpha=alpha, depth=depth, threads=4)
    assert np.array_equal(res["adj"], ref["adj"])
    assert res["sepsets"] == ref["sepsets"]
    assert st["tests"] == ref["stats"]["tests"]


def test_constant_column_in_skeleton(eng):
    """A variable with a single observed state is independent of everything (df 0)."""
    raw, _, _ = F.generate(n_nodes=10, n_samples=4000, seed=33, n_edges=12, max_indegree=3, card=(2, 4))
    raw[4, :] = 7
    cols, card = O.relabel(raw)
    eng.upload(raw)
    st = eng.pc_skeleton().to_dict()
    res = eng.result()
    ref = O.pc_skeleton(cols, card, threads=4)
    assert not res["adj"][4].any()
    assert np.array_equal(res["adj"], ref["adj"]) and res["sepsets"] == ref["sepsets"]
    assert st["tests"] == ref["stats"]["tests"]


_DAG_PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include "fastpgm_gb300_cxx.h"
int main(int argc, char **argv) {
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(argv[1], true, 0);
    Network *net = new Network(true);
    PCStable *pc = new PCStable(net, 0.05);
    pc->StructLearnCompData(d, 1, 1, true, atoi(argv[2]) != 0, false, "", 0);
    printf("nodes %d\n", net->num_nodes);
    for (auto &e : net->vec_edges)
        printf("%d %d %d\n", e.node1->GetNodeIndex(), e.node2->GetNodeIndex(), e.end_point2 == ARROW ? 1 : 0);
    return 0;
}
"""


@pytest.mark.parametrize("add_root", [0, 1])
def test_cxx_dag_and_root_options(tmp_path, add_root):
    """StructLearnCompData(dag=true) directs the undirected records that lead the edge list
    (randomly, as the reference's DirectLeftEdges does, stopping at the first directed record)
    so the graph is acyclic over the learned skeleton; add_root adds a ROOT node as the parent
    of each connected sub-graph's root (StructureLearning.cpp:110-240)."""
    raw, _, _ = F.make_config("c1")
    csv = str(tmp_path / "c1.csv")
    F.write_csv(csv, raw)
    src = tmp_path / "dag.cpp"
    src.write_text(_DAG_PROGRAM)
    exe = str(tmp_path / "dag")
    libdir = os.path.dirname(F.LIB_PATH)
    from conftest import ROOT
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe, "-L",
                    libdir, "-lfastpgm_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([exe, csv, str(add_root)], capture_output=True, text=True, check=True).stdout.splitlines()
    n = int([l for l in out if l.startswith("nodes")][0].split()[1])
    edges = [tuple(map(int, l.split())) for l in out if l and l[0].isdigit()]
    assert edges[0][2] == 1  # no undirected record leads any more
    n0 = raw.shape[0]
    cols, card = O.relabel(raw)
    ref = O.pc_skeleton(cols, card, threads=4)
    skel = {(min(a, b), max(a, b)) for a, b, _ in edges if a < n0 and b < n0}
    assert skel == {(i, j) for i in range(n0) for j in range(i + 1, n0) if ref["adj"][i, j]}
    # acyclic: Kahn's algorithm consumes every node
    import collections
    arcs = {(a, b) for a, b, d in edges if d == 1}
    indeg = collections.Counter(b for _, b in arcs)
    children = collections.defaultdict(list)
    for a, b in arcs:
        children[a].append(b)
    ready = [v for v in range(n) if indeg[v] == 0]
    seen = 0
    while ready:
        v = ready.pop()
        seen += 1
        for c in children[v]:
            indeg[c] -= 1
            if indeg[c] == 0:
                ready.append(c)
    assert seen == n
    if add_root:
        assert n == n0 + 1 and any(a == n0 for a, _, _ in edges)
    else:
        assert n == n0


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_device_driven_waves_match_host_driven(monkeypatch, name):
    """Levels >= 1 run as one CUDA graph each (a WHILE conditional node over the wave body,
    the tail kernel deciding on the device whether another wave runs); FPGM_GRAPH=0 drives
    every wave from the host.  Same skeleton, separating sets, and per-level test, executed
    test and wave counts."""
    raw, depth, _ = F.make_config(name)
    out = {}
    for graph in ("1", "0"):
        monkeypatch.setenv("FPGM_GRAPH", graph)
        with F.Engine(0) as e:
            e.upload(raw)
            st = e.pc_skeleton(depth=depth).to_dict()
            out[graph] = (st, e.result())
    (sg, rg), (sh, rh) = out["1"], out["0"]
    assert np.array_equal(rg["adj"], rh["adj"]) and rg["sepsets"] == rh["sepsets"]
    for k in ("tests", "tests_executed", "edges_after", "waves"):
        assert sg[k] == sh[k], k


def test_online_autotuner_times_both_tier2_methods(monkeypatch):
    """The online autotuner times the partition kernel and the global strata hash per
    (samples, |Z|, cells/samples) bucket on the tier-2 tests a skeleton runs (FPGM_WIDE=0 so
    that no wave hands its tests over wholesale): after two skeletons of a 70,000-sample
    dataset with 6-9 states it has timed tests both ways, and the skeleton equals the oracle's
    whichever method each test took; FPGM_TUNE=0 times nothing."""
    raw, _, _ = F.generate(n_nodes=12, n_samples=70000, seed=72, n_edges=30, max_indegree=5, card=(6, 10))
    cols, card = O.relabel(raw)
    ref = O.pc_skeleton(cols, card, threads=16)
    for tune, timed in (("1", True), ("0", False)):
        monkeypatch.setenv("FPGM_WIDE", "0")
        monkeypatch.setenv("FPGM_TUNE", tune)
        with F.Engine(0) as e:
            e.upload(raw)
            for _ in range(2):
                st = e.pc_skeleton().to_dict()
                res = e.result()
                assert np.array_equal(res["adj"], ref["adj"]) and res["sepsets"] == ref["sepsets"]
        assert (st["tune_timed"] > 0) == timed and (st["tune_buckets"] > 0) == timed


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_large_warp_slices_match_reference(monkeypatch, tmp_path, name):
    """The warp tier with 12 KB slices (FPGM_WARP_SLICE=3072: 2 CTAs per SM, tables up to
    3,040 ints; the default is 8 KB slices and 3 CTAs per SM) gives the reference's
    separating sets and CPDAG."""
    monkeypatch.setenv("FPGM_WARP_SLICE", "3072")
    raw, depth, _ = F.make_config(name)
    with F.Engine(0) as e:
        e.upload(raw)
        e.pc_skeleton(depth=depth)
        res = e.result()
    assert res["sepsets"] == read_sepsets(os.path.join(GOLDEN, name + "_sepsets"))
    n = raw.shape[0]
    assert struct_of(tmp_path, ["V%d" % i for i in range(n)], res) == open(os.path.join(GOLDEN, name + "_struct")).read()


@pytest.mark.parametrize("env", [{}, {"FPGM_OVF_SKIP": "0"}, {"FPGM_STAGE_REC": "64"}, {"FPGM_STAGE_REC": "1024"},
                                 {"FPGM_LIVE": "0"}, {"FPGM_LIVE_FRAC": "1.01", "FPGM_LIVE_MIN_LEVEL": "2"},
                                 {"FPGM_LIVE_FRAC": "1.01", "FPGM_LIVE_MIN_LEVEL": "2", "FPGM_STAGE_REC": "512"}])
def test_tier2_paths_match_oracle_over_repeated_skeletons(monkeypatch, env):
    """Tier 2 on a 70,000-sample dataset with 6-9 states, three skeletons on one engine (the
    autotuner and the shared-hash overflow record carry over from one to the next, so later
    skeletons skip the shared-hash attempt where it overflowed before): the default, the
    attempt never skipped (FPGM_OVF_SKIP=0), the staged super-partitions capped at 64 or
    1,024 records (FPGM_STAGE_REC; at 64 nearly every partition is counted from its records
    in global memory instead), no contributing-sample bitmaps (FPGM_LIVE=0), and bitmaps
    written at every level from level 2 (FPGM_LIVE_FRAC above 1), also with partitions
    beyond the staged cap (whose tests then leave their bitmaps out).  Every skeleton equals
    the oracle's, test counts included."""
    raw, _, _ = F.generate(n_nodes=12, n_samples=70000, seed=72, n_edges=30, max_indegree=5, card=(6, 10))
    cols, card = O.relabel(raw)
    ref = O.pc_skeleton(cols, card, threads=16)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with F.Engine(0) as e:
        e.upload(raw)
        for _ in range(3):
            st = e.pc_skeleton().to_dict()
            res = e.result()
            assert np.array_equal(res["adj"], ref["adj"]) and res["sepsets"] == ref["sepsets"]
            assert st["tests"] == ref["stats"]["tests"]


def test_bitmaps_follow_a_larger_dataset_in_the_same_engine(monkeypatch):
    """Contributing-sample bitmaps written at every level from level 2 (FPGM_LIVE_FRAC above
    1), in one engine that learns a 20,000-sample dataset and then a 70,000-sample one: the
    bitmap pools are remade for the larger sample count, and both skeletons equal the oracle's."""
    monkeypatch.setenv("FPGM_LIVE_FRAC", "1.01")
    monkeypatch.setenv("FPGM_LIVE_MIN_LEVEL", "2")
    with F.Engine(0) as e:
        for S, seed in ((20000, 73), (70000, 72)):
            raw, _, _ = F.generate(n_nodes=12, n_samples=S, seed=seed, n_edges=30, max_indegree=5, card=(6, 10))
            cols, card = O.relabel(raw)
            ref = O.pc_skeleton(cols, card, threads=16)
            e.upload(raw)
            for _ in range(2):
                st = e.pc_skeleton().to_dict()
                res = e.result()
                assert np.array_equal(res["adj"], ref["adj"]) and res["sepsets"] == ref["sepsets"], S
                assert st["tests"] == ref["stats"]["tests"], S
