"""GPU maximum-likelihood parameter learning for a known DAG (the reference's job -j 1,
ParameterLearning::LearnParamsKnowStructCompData) against the oracle, which the CPU tests
pin to the reference's own ParameterLearning bit for bit."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
import fastpgm_gb300 as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = F.Engine(0)
    yield e
    e.close()


def _check_all(eng, raw, par, alpha):
    cols, card = O.relabel(raw)
    eng.upload(raw)
    parents = [par[v] for v in range(raw.shape[0])]
    got = eng.mle_cpts(parents, alpha=alpha)
    exp = O.mle_cpts(cols, card, parents, alpha=alpha)
    for v, (g, o) in enumerate(zip(got, exp)):
        assert g.shape == o.shape and np.array_equal(g, o), v
    return got


@pytest.mark.parametrize("alpha", [0, 1, 2])
def test_true_dag_tables_c1(eng, alpha):
    raw, _, par = F.generate(n_nodes=37, n_samples=5000, seed=1, n_edges=46, max_indegree=4, card=(2, 4))
    _check_all(eng, raw, par, alpha)


@pytest.mark.parametrize("name", ["c2", "c4"])
def test_true_dag_tables_configs(eng, name):
    """c2 (50,000 samples) and c4 (1,041 nodes, 100,000 samples, tables to 21^4) with the
    generating DAG: shared-memory and global-memory counting."""
    spec = dict(F.CONFIGS[name])
    spec.pop("depth")
    raw, _, par = F.generate(**spec)
    got = _check_all(eng, raw, par, 1)
    if name == "c4":
        assert max(len(g) for g in got) > 24576  # counted in global memory


def test_wide_parent_sets(eng):
    raw, _, par = F.generate(n_nodes=16, n_samples=20000, seed=9, n_edges=30, max_indegree=5, card=(6, 9))
    got = _check_all(eng, raw, par, 1)
    assert max(len(g) for g in got) > 24576


def test_several_datasets(eng):
    jobs = F.c5_jobs(seed=71, n_jobs=3)
    data, pars = [], []
    for j in jobs:
        j = dict(j)
        j.pop("depth")
        j["n_samples"] = min(j["n_samples"], 20000)
        raw, _, par = F.generate(**j)
        data.append(raw)
        pars.append(par)
    eng.upload_jobs(data)
    parents = []
    for raw, par, base in zip(data, pars, eng.job_offsets[:-1]):
        parents += [[int(p) + int(base) for p in par[v] if p >= 0] for v in range(raw.shape[0])]
    got = eng.mle_cpts(parents, alpha=1)
    for raw, par, base in zip(data, pars, eng.job_offsets[:-1]):
        cols, card = O.relabel(raw)
        exp = O.mle_cpts(cols, card, [par[v] for v in range(raw.shape[0])], alpha=1)
        for v in range(raw.shape[0]):
            assert np.array_equal(got[int(base) + v], exp[v])


def test_invalid_parent_lists(eng):
    raw, _, par = F.generate(n_nodes=6, n_samples=500, seed=3, n_edges=5, max_indegree=2, card=(2, 3))
    eng.upload(raw)
    L = F.load()
    i64 = ctypes.POINTER(ctypes.c_int64)
    toff = np.zeros(7, dtype=np.int64)
    for off, flat in (([0, 2, 2, 2, 2, 2, 2], [3, 1]),   # not ascending
                      ([0, 1, 1, 1, 1, 1, 1], [0]),      # a node its own parent
                      ([0, 1, 1, 1, 1, 1, 1], [9])):     # out of range
        off = np.array(off, dtype=np.int32)
        flat = np.array(flat, dtype=np.int32)
        rc = L.fpgm_mle_cpts(eng._h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                             flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 1, toff.ctypes.data_as(i64), None)
        assert rc == F.FPGM_ERR_INVALID


_PROGRAM = r"""
#include <cstdlib>
#include <fstream>
#include "fastpgm_gb300_cxx.h"
int main(int argc, char **argv) {
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(argv[1], true, 0);
    Network *net = new Network(true);
    PCStable pc(net, 0.05);     // only to build the nodes from the dataset
    pc.AssignNodeInformation(d);
    std::ifstream in(argv[2]);
    int p, c;
    while (in >> p >> c) {
        net->FindNodePtrByIndex(c)->set_parent_indexes.insert(p);
        net->FindNodePtrByIndex(p)->set_children_indexes.insert(c);
    }
    ParameterLearning pl(net);
    pl.LearnParamsKnowStructCompData(d, atoi(argv[3]), true, argv[4], 0);
    return 0;
}
"""


def test_cxx_parameter_learning_reproduces_reference_file(tmp_path):
    """The C++ drop-in ParameterLearning writes, for c1's generating DAG, the same file the
    reference's own ParameterLearning + SaveBNParameter wrote (tests/golden/c1_param_alpha1)."""
    import os
    import subprocess
    from conftest import GOLDEN, ROOT
    raw, _, _ = F.make_config("c1")
    csv = str(tmp_path / "c1.csv")
    F.write_csv(csv, raw)
    src = tmp_path / "pl.cpp"
    src.write_text(_PROGRAM)
    exe = str(tmp_path / "pl")
    libdir = os.path.dirname(F.LIB_PATH)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe,
                    "-L", libdir, "-lfastpgm_gb300", "-Wl,-rpath," + libdir], check=True)
    out = str(tmp_path / "param")
    subprocess.run([exe, csv, os.path.join(GOLDEN, "c1_dag"), "1", out], check=True, capture_output=True)
    assert open(out).read() == open(os.path.join(GOLDEN, "c1_param_alpha1")).read()
