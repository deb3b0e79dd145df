"""The CPU oracle pinned against the reference's own outputs (golden fixtures).

Fixtures come from the reference's PC-stable code compiled as-is (oracle/_ref,
regenerated by tests/golden/make_golden.py), plus the reference's shipped golden
CPDAG dataset/alarm/alarm_s5000_struct.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, read_sepsets, read_tests, tiny_table_cases
from oracle import oracle as O
import fastpgm_gb300 as F


def test_igamma_matches_scipy():
    sp = pytest.importorskip("scipy.special")
    import ctypes
    # the oracle header is compiled into liboracle; check the restatement through the tests API
    rng = np.random.default_rng(0)
    for _ in range(400):
        a = float(10 ** rng.uniform(-0.3, 4))
        x = float(a * 10 ** rng.uniform(-1.5, 0.7))
        # p = 1 - P(a, x): build a 2 x 2k table would be indirect; use the C header through a tiny shim
        ref = sp.gammainc(a, x)
        got = _igamma_p(a, x)
        assert abs(got - ref) <= 1e-12 + 1e-10 * ref, (a, x, got, ref)


def _igamma_p(a, x):
    import ctypes
    import subprocess
    import tempfile
    global _IG
    try:
        return _IG(a, x)
    except NameError:
        pass
    d = tempfile.mkdtemp()
    src = os.path.join(d, "ig.c")
    with open(src, "w") as f:
        f.write('#include "igamma.h"\ndouble ig(double a, double x) { return oracle_igamma_p(a, x); }\n')
    so = os.path.join(d, "ig.so")
    subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-I", os.path.dirname(O.__file__), src, "-o", so, "-lm"])
    lib = ctypes.CDLL(so)
    lib.ig.restype = ctypes.c_double
    lib.ig.argtypes = [ctypes.c_double, ctypes.c_double]
    _IG = lib.ig
    return _IG(a, x)


@pytest.mark.parametrize("which", ["alarm", "c1"])
def test_oracle_ci_tests_match_reference_vectors(which, alarm):
    if which == "alarm":
        _, cols, card = alarm
    else:
        import fastpgm_gb300 as F
        raw, _, _ = F.make_config("c1")
        cols, card = O.relabel(raw)
    gold = read_tests(os.path.join(GOLDEN, which + "_tests.txt"))
    by_d = {}
    for g in gold:
        by_d.setdefault(len(g[2]), []).append(g)
    for d, items in by_d.items():
        tests = np.array([[x, y, *z] for x, y, z, *_ in items], dtype=np.int32)
        res = O.ci_tests(cols, card, tests, d, threads=4)
        for g, r in zip(items, res):
            x, y, z, h, df, g2, p, ind = g
            assert r.table_hash == h and r.df == df and r.independent == ind, g
            assert abs(r.g2 - g2) <= 1e-9 * max(1.0, abs(g2)), g
            assert abs(r.p_value - p) <= 1e-12, g


def test_oracle_skeleton_alarm(alarm):
    _, cols, card = alarm
    r = O.pc_skeleton(cols, card, threads=4)
    assert r["sepsets"] == read_sepsets(os.path.join(GOLDEN, "alarm_sepsets"))
    # per-level deterministic test counts of the reference at one thread
    assert r["stats"]["tests"] == [666, 3579, 828, 118, 15]
    assert r["stats"]["edges_after"] == [262, 67, 46, 44, 44]


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_generator_is_deterministic_and_oracle_matches(name):
    import fastpgm_gb300 as F
    meta = json.load(open(os.path.join(GOLDEN, name + "_meta.json")))
    raw, depth, _ = F.make_config(name)
    assert list(raw.shape) == meta["shape"]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == meta["sha256"]
    cols, card = O.relabel(raw)
    r = O.pc_skeleton(cols, card, depth=depth, threads=8)
    assert r["sepsets"] == read_sepsets(os.path.join(GOLDEN, name + "_sepsets"))


def test_relabel_first_appearance():
    raw = np.array([[3, 3, 1, 7, 1, 3], [0, 0, 0, 0, 0, 0]], dtype=np.uint8)
    cols, card = O.relabel(raw)
    assert cols.tolist() == [[0, 0, 1, 2, 1, 0], [0] * 6]
    assert card.tolist() == [3, 1]


@pytest.mark.skipif(not O.ref_available(), reason="reference-built driver needs the reference tree")
def test_reference_driver_reproduces_shipped_golden(tmp_path):
    O.ref_pc(os.path.join(O.REFERENCE_TREE, "dataset", "alarm", "alarm_s5000"), str(tmp_path / "a"))
    got = open(tmp_path / "a_struct").read()
    assert got == open(os.path.join(GOLDEN, "alarm_s5000_struct")).read()


@pytest.mark.skipif(not O.ref_available(), reason="reference-built driver needs the reference tree")
def test_sparse_oracle_path_matches_reference_bit_for_bit(tmp_path):
    """Tables above 2^24 cells are counted from sorted keys; G^2 must equal the reference's dense loop."""
    import subprocess
    import fastpgm_gb300 as F
    rng = np.random.default_rng(2)
    S = 20000
    raw = np.stack([rng.integers(0, 9, S), rng.integers(0, 8, S)] + [rng.integers(0, 64, S) for _ in range(3)])
    raw[1] = (raw[1] + (raw[0] > 6)) % 8
    raw = raw.astype(np.uint8)
    csv = str(tmp_path / "big.csv")
    F.write_csv(csv, raw)
    tin, tout = str(tmp_path / "t.txt"), str(tmp_path / "o.txt")
    with open(tin, "w") as f:
        f.write("0 1 3 2 3 4\n")
    subprocess.check_call([O.REF_DRIVER, "tests", csv, "0.05", tin, tout])
    h, df, g2, p, ind = open(tout).read().split()
    cols, card = O.relabel(raw)
    r = O.ci_tests(cols, card, np.array([[0, 1, 2, 3, 4]], dtype=np.int32), 3, threads=1)[0]
    assert r.cells > (1 << 24) and r.table_hash == 0
    assert r.df == int(df) and r.independent == int(ind)
    assert r.g2 == float(g2) and r.p_value == float(p)


def test_wilson_hilferty_router_bound():
    """The engine routes tests with df > 32768 by the Wilson-Hilferty tail with a 1e-5 margin;
    its error against the exact incomplete gamma must stay far below that margin."""
    sp = pytest.importorskip("scipy.special")
    st = pytest.importorskip("scipy.stats")
    for k in (32769, 50000, 1e5, 1e6):
        xs = st.chi2.ppf(np.linspace(1e-6, 1 - 1e-6, 4001), k)
        exact = sp.gammaincc(k / 2, xs / 2)
        v = 2 / (9 * k)
        wh = 0.5 * sp.erfc((np.cbrt(xs / k) - (1 - v)) / np.sqrt(v) / np.sqrt(2))
        assert np.abs(wh - exact).max() < 1e-6
        assert st.chi2.pdf(xs, k).max() < 0.3 / np.sqrt(k)


@pytest.mark.skipif(not O.ref_available(), reason="reference-built driver needs the reference tree")
@pytest.mark.parametrize("alpha", [0, 1, 3])
def test_mle_oracle_matches_reference_parameter_learning(tmp_path, alpha):
    """The oracle's maximum-likelihood tables equal the reference's own
    ParameterLearning::LearnParamsKnowStructCompData bit for bit, for the true DAG of a
    generated network (nodes with 0 to 4 parents)."""
    raw, _, par = F.generate(n_nodes=37, n_samples=5000, seed=1, n_edges=46, max_indegree=4, card=(2, 4))
    csv = str(tmp_path / "d.csv")
    F.write_csv(csv, raw)
    edges = [(int(p), c) for c in range(par.shape[0]) for p in par[c] if p >= 0]
    ref = O.ref_mle(csv, alpha, edges, str(tmp_path))
    cols, card = O.relabel(raw)
    got = O.mle_cpts(cols, card, [par[c] for c in range(par.shape[0])], alpha=alpha)
    assert any(len(v) > 3 for v, _ in ref.values())
    for v in range(raw.shape[0]):
        rel, pots = ref[v]
        assert rel[0] == v and rel[1:] == sorted(int(p) for p in par[v] if p >= 0)
        assert np.array_equal(got[v], pots), v


@pytest.mark.parametrize("case", tiny_table_cases(), ids=lambda c: c[0])
def test_oracle_known_answers_on_tiny_tables(case):
    name, raw, d, g2, df, p = case
    cols, card = O.relabel(raw)
    r = O.ci_tests(cols, card, np.array([list(range(2 + d))], dtype=np.int32), d, threads=1)[0]
    assert r.df == df and abs(r.g2 - g2) < 1e-12 and abs(r.p_value - p) < 1e-12
    assert r.independent == (p > 0.05)


@pytest.mark.parametrize("name", ["c3", "c4", "c5"])
def test_full_size_fixtures_describe_this_hosts_data(name):
    """The full-size fixtures (oracle digests at the c3/c4/c5 sizes, checked against the GPU
    engine in test_gpu_fullsize.py) were made from the bytes the seeded sampler gives here."""
    from fastpgm_gb300 import configs as C
    with open(os.path.join(GOLDEN, "full_%s.json" % name)) as f:
        fx = json.load(f)
    if name == "c5":
        data, depth = C.make_jobs(C.c5_jobs(), generate=O.generate)
    else:
        raw, depth, _ = C.make_config(name, generate=O.generate)
        data = [raw]
    assert depth == fx["depth"] and len(data) == len(fx["jobs"])
    for raw, job in zip(data, fx["jobs"]):
        if job is None:
            continue
        assert O.sha256(raw) == job["sha256"]
        assert list(raw.shape) == job["shape"]
        assert len(job["tests"]) == len(job["edges_after"]) >= 1
