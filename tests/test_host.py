"""Host-side checks that need no GPU: the C-ABI library loads and exports every
declared symbol, the host orientation reproduces the reference's CPDAG files,
the command line and the Python binding parse like the reference's."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, read_sepsets, sepset_arrays
from oracle import oracle as O
import fastpgm_gb300 as F


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            # declarations only: a return type at the start of the line, then the name
            names |= set(re.findall(r"^(?:int|const char \*)\s*(fpgm_[a-z0-9_]+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = F.load()
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", F.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fpgm_\w+)", out))
    assert names <= exported, names - exported


def test_ctypes_structs_match_the_c_header(tmp_path):
    """The Python binding's structures have the C header's sizes and field offsets."""
    checks = {"fpgm_pc_stats": (F.PCStats, ["count_ms", "large_ms", "span_ms", "total_ms", "large_bytes"]),
              "fpgm_ci_result": (F.CIResult, ["df", "g2", "p_value", "path"]),
              "fpgm_gen_spec": (F.GenSpec, ["n_samples", "seed"])}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fastpgm_gb300.h"', "int main(void) {"]
    for c, (_, fields) in checks.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (c, c))
        for f in fields:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (c, f, c, f))
    lines.append("return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True)
               .stdout.splitlines())
    for c, (cls, fields) in checks.items():
        assert int(got[c]) == ctypes.sizeof(cls), c
        for f in fields:
            assert int(got["%s.%s" % (c, f)]) == getattr(cls, f).offset, (c, f)


def _orient_struct(tmp_path, names, adj, seps):
    removed, off, vs = sepset_arrays(seps)
    edges = F.orient_cpdag(adj, removed, off, vs)
    p = str(tmp_path / "s_struct")
    F.write_struct(p, names, edges, int(adj.sum()) // 2)
    return open(p).read()


def test_orientation_reproduces_alarm_golden(tmp_path, alarm):
    names, cols, card = alarm
    r = O.pc_skeleton(cols, card, threads=4)
    got = _orient_struct(tmp_path, names, r["adj"], r["sepsets"])
    assert got == open(os.path.join(GOLDEN, "alarm_s5000_struct")).read()


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_orientation_reproduces_reference_cpdag(tmp_path, name):
    seps = read_sepsets(os.path.join(GOLDEN, name + "_sepsets"))
    raw, depth, spec = F.make_config(name)
    n = raw.shape[0]
    adj = np.ones((n, n), dtype=np.uint8) - np.eye(n, dtype=np.uint8)
    for a, b in seps:
        adj[a, b] = adj[b, a] = 0
    got = _orient_struct(tmp_path, ["V%d" % i for i in range(n)], adj, seps)
    assert got == open(os.path.join(GOLDEN, name + "_struct")).read()


def _collider_csv(path, S=4000, seed=3):
    """a, c independent; b depends on both -> PC finds a -> b <- c; d independent of all."""
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2, S)
    c = rng.integers(0, 2, S)
    b = (a | c) ^ (rng.random(S) < 0.05)
    e = rng.integers(0, 3, S)
    cols = np.stack([a, b, c, e]).astype(np.uint8)
    F.write_csv(path, cols)
    return cols


@pytest.mark.skipif(not O.ref_available(), reason="reference-built driver needs the reference tree")
def test_dag_branch_of_struct_writer_matches_reference(tmp_path):
    csv = str(tmp_path / "col.csv")
    raw = _collider_csv(csv)
    O.ref_pc(csv, str(tmp_path / "ref"))
    cols, card = O.relabel(raw)
    r = O.pc_skeleton(cols, card)
    got = _orient_struct(tmp_path, ["V%d" % i for i in range(4)], r["adj"], r["sepsets"])
    ref = open(tmp_path / "ref_struct").read()
    assert "->" in ref
    assert got == ref


def test_engine_create_without_gpu_reports_error():
    import ctypes
    lib = F.load()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    rc = lib.fpgm_engine_create(0, ctypes.byref(h))
    assert rc != 0
    assert lib.fpgm_last_error()


def test_cli_help_and_rejected_jobs():
    out = subprocess.run([F.CLI_PATH, "-h"], capture_output=True, text=True)
    assert out.returncode == 0 and "-j & -m" in out.stdout
    out = subprocess.run([F.CLI_PATH, "-j", "2", "-m", "0"], capture_output=True, text=True)
    assert out.returncode == 1 and "Only -j 0" in out.stdout and "-j 1" in out.stdout
    out = subprocess.run([F.CLI_PATH, "-v", "1"], capture_output=True, text=True)
    assert "Unrecognized option -v" in out.stdout  # the reference does not parse -v either


def test_generator_rejects_bad_spec():
    with pytest.raises(F.FpgmError):
        F.generate(n_nodes=1, n_samples=10, seed=1)
    with pytest.raises(F.FpgmError):
        F.generate(n_nodes=5, n_samples=10, seed=1, card=(1, 3))


def test_python_binding_module_signature():
    from fastpgm_gb300 import cmake_example
    import inspect
    params = list(inspect.signature(cmake_example.BNSL_PCStable).parameters)
    assert params == ["verbose", "n_threads", "group_size", "alpha", "ref_net", "train_set", "save_struct"]


def _write_bif(path, card, parents):
    """A minimal BIF file of a DAG (uniform tables), in the layout the reference's
    CustomNetwork::LoadBIFFile reads."""
    import itertools
    n = len(card)
    lines = ["network unknown {", "}"]
    for v in range(n):
        states = ", ".join("s%d" % k for k in range(card[v]))
        lines += ["variable V%d {" % v, "  type discrete [ %d ] { %s };" % (card[v], states), "}"]
    for v in range(n):
        ps = [int(p) for p in parents[v] if p >= 0]
        row = ", ".join(["%.4f" % (1.0 / card[v])] * card[v]) + ";"
        if not ps:
            lines += ["probability ( V%d ) {" % v, "  table " + row, "}"]
            continue
        lines.append("probability ( V%d | %s ) {" % (v, ", ".join("V%d" % p for p in ps)))
        for cfg in itertools.product(*[range(card[p]) for p in ps]):
            lines.append("  (%s) %s" % (", ".join("s%d" % c for c in cfg), row))
        lines.append("}")
    open(path, "w").write("\n".join(lines) + "\n")


def _learned_edges(cols, card):
    r = O.pc_skeleton(cols, card, threads=8)
    removed, off, vs = sepset_arrays(r["sepsets"])
    return F.orient_cpdag(r["adj"], removed, off, vs)


def test_shd_of_a_dag_against_its_own_bif(tmp_path):
    """A learned DAG (first edge directed: no CPDAG conversion) scores 0 against itself, and
    one missing arc or one reversed arc cost 1 each."""
    _, card, par = F.generate(n_nodes=12, n_samples=100, seed=5, n_edges=14, max_indegree=3, card=(2, 3))
    bif = str(tmp_path / "g.bif")
    _write_bif(bif, card, par)
    arcs = [(int(p), c, 1) for c in range(12) for p in par[c] if p >= 0]
    assert F.shd_bif(bif, 12, arcs) == 0
    assert F.shd_bif(bif, 12, arcs[:-1]) == 1
    a, b, _ = arcs[-1]
    assert F.shd_bif(bif, 12, arcs[:-1] + [(b, a, 1)]) == 1


@pytest.mark.skipif(not O.ref_available(), reason="reference-built driver needs the reference tree")
def test_shd_matches_reference_comparison(tmp_path):
    """BNSL_PCStable's SHD report: the learned CPDAG against the reference network, equal to
    the reference's own CustomNetwork::LoadBIFFile + BNSLComparison::GetSHD -- on alarm
    (its shipped alarm.bif) and on c1 (its generating DAG written as BIF)."""
    ref_root = os.path.join(O.REFERENCE_TREE, "dataset", "alarm") + os.sep
    cases = [(ref_root + "alarm_s5000", ref_root + "alarm.bif", None)]
    raw, card, par = F.generate(n_nodes=37, n_samples=5000, seed=1, n_edges=46, max_indegree=4, card=(2, 4))
    c1_csv, c1_bif = str(tmp_path / "c1.csv"), str(tmp_path / "c1.bif")
    F.write_csv(c1_csv, raw)
    _write_bif(c1_bif, card, par)
    cases.append((c1_csv, c1_bif, raw))
    for csv, bif, raw in cases:
        out = subprocess.run([O.REF_DRIVER, "shd", csv, "0.05", bif], capture_output=True, text=True, check=True)
        ref = int(re.search(r"SHD = (\d+)", out.stdout).group(1))
        if raw is None:
            names, cols, cd = O.read_csv_columns(csv)
        else:
            cols, cd = O.relabel(raw)
        assert F.shd_bif(bif, cols.shape[0], _learned_edges(cols, cd)) == ref


_LOADER = r"""
#include <cstdio>
#include "fastpgm_gb300_cxx.h"
int main(int argc, char **argv) {
    Dataset d;
    d.LoadCSVTrainingData(argv[1], true, 0);
    FILE *f = fopen(argv[2], "wb");
    fprintf(f, "%d %d\n", d.num_vars, d.num_instance);
    for (auto &n : d.vec_var_names) fprintf(f, "%s\n", n.c_str());
    for (int c : d.num_of_possible_values_of_disc_vars) fprintf(f, "%d\n", c);
    fwrite(d.columns.data(), 1, d.columns.size(), f);
    fclose(f);
    return 0;
}
"""


def test_parallel_csv_loader_matches_first_appearance_ids(tmp_path):
    """The C++ drop-in Dataset::LoadCSVTrainingData (parallel parse) gives the reference's
    first-appearance ids and cardinalities: string values, CRLF line ends, blank lines,
    values whose first appearance falls late in the file (other threads' rows)."""
    rng = np.random.default_rng(3)
    n, S = 7, 20000
    vals = [["a", "bb", "c c", "-1"], ["x"], ["0", "1"], ["u%d" % k for k in range(40)], ["p", "q", "r"],
            ["7", "8"], ["late", "early"]]
    cols = []
    for v in range(n):
        idx = rng.integers(0, len(vals[v]), S)
        cols.append([vals[v][i] for i in idx])
    cols[6] = ["early"] * (S - 3) + ["late"] * 3  # second value first appears at the end
    path = tmp_path / "d.csv"
    with open(path, "w", newline="") as f:
        f.write(",".join("N%d" % v for v in range(n)) + "\r\n")
        for s in range(S):
            f.write(",".join(cols[v][s] for v in range(n)) + ("\r\n" if s % 3 else "  \n"))
            if s % 5000 == 0:
                f.write("\n")
    names, ref_cols, ref_card = O.read_csv_columns(str(path))
    src = tmp_path / "load.cpp"
    src.write_text(_LOADER)
    exe = str(tmp_path / "load")
    libdir = os.path.dirname(F.LIB_PATH)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe, "-L",
                    libdir, "-lfastpgm_gb300", "-Wl,-rpath," + libdir], check=True)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(path), str(out)], check=True, capture_output=True)
    data = out.read_bytes()
    lines = data.split(b"\n", 1 + 2 * n)
    nv, ni = map(int, lines[0].split())
    assert (nv, ni) == (n, S)
    assert [l.decode() for l in lines[1:1 + n]] == names
    assert [int(l) for l in lines[1 + n:1 + 2 * n]] == list(ref_card)
    got = np.frombuffer(lines[-1], dtype=np.uint8).reshape(n, S)
    assert np.array_equal(got, ref_cols)


def test_autotuner_bucket_keys():
    """tune.tune_index mirrors the engine's tune_index (ci_kernels.cuh): sample buckets from
    12,500 doubling, |Z| 1..12, cells/samples in powers of 4 from 4."""
    from fastpgm_gb300 import tune
    assert tune.tune_index(12499, 1, 10) == (0, 0, 0)
    assert tune.tune_index(12500, 1, 12500 * 4) == (1, 0, 1)
    assert tune.tune_index(50000, 6, 50000 * 100) == (3, 5, 3)
    assert tune.tune_index(10 ** 7, 40, 1e30) == (5, 11, 5)
    assert tune.tune_index(100000, 0, 1) == (4, 0, 0)


def test_top_level_cmake_example_module():
    """`import cmake_example` -- the first line of the reference's python/pyfastpgm.py --
    resolves to this repository's drop-in when the repository is on PYTHONPATH."""
    code = "import cmake_example as f; print(f.BNSL_PCStable.__module__, callable(f.BNL_PCStable))"
    env = dict(os.environ, PYTHONPATH=ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd="/", env=env)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["fastpgm_gb300.cmake_example", "True"]
