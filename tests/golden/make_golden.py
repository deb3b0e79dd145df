"""Regenerates the committed golden fixtures from the reference's own PC-stable code.

Needs the reference tree (FastPGM; $FASTPGM_REFERENCE, default /root/reference) and the reference-built
driver (oracle/Makefile `ref` target).  Writes, under tests/golden/:

  alarm_s5000.npz        the reference's shipped alarm_s5000 dataset, as the reference
                         loader sees it: uint8 ids by first appearance + names
  alarm_s5000_struct     the reference's shipped golden CPDAG (dataset/alarm/alarm_s5000_struct)
  alarm_sepsets          sepsets of the reference run (ref_driver pc)
  <cfg>_struct           reference CPDAG on the seeded synthetic config (c1, c2)
  <cfg>_sepsets          reference sepsets on it
  <cfg>_meta.json        sha256 of the generated raw columns, shape, reference test count
  <set>_tests.txt        per-test golden vectors from the reference's IndependenceTest and
                         Counts2D/Counts3D: "x y d z.. | hash df g2 p indep"
  c1_dag                 the generating DAG of c1 as "parent child" lines
  c1_param_alpha1        the reference's ParameterLearning (Laplace alpha 1) for that DAG,
                         written by its own SaveBNParameter
  c1_bnl_param           BNL_PCStable's parameter file on c1: the reference's ParameterLearning
                         (alpha 1) on the graph its PC-stable learned

Run:  python tests/golden/make_golden.py [--mle-only]
"""
import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import fastpgm_gb300 as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = O.REFERENCE_TREE


def sample_tests(n, card, rng, count, dmax):
    tests = []
    for _ in range(count):
        d = int(rng.integers(0, dmax + 1))
        vs = rng.choice(n, size=2 + d, replace=False)
        tests.append((int(vs[0]), int(vs[1]), [int(v) for v in vs[2:]]))
    return tests


def ref_tests(csv, tests, out_path):
    tmp = tempfile.mkdtemp()
    try:
        tin = os.path.join(tmp, "t.txt")
        tout = os.path.join(tmp, "o.txt")
        with open(tin, "w") as f:
            for x, y, z in tests:
                f.write("%d %d %d %s\n" % (x, y, len(z), " ".join(map(str, z))))
        import subprocess
        subprocess.check_call([O.REF_DRIVER, "tests", csv, "0.05", tin, tout])
        with open(tout) as f:
            res = [l.strip() for l in f if l.strip()]
        with open(out_path, "w") as f:
            for (x, y, z), r in zip(tests, res):
                f.write("%d %d %d %s | %s\n" % (x, y, len(z), " ".join(map(str, z)), r))
    finally:
        shutil.rmtree(tmp)


def mle_golden():
    """c1's true DAG and the reference's parameter file for it."""
    spec = dict(F.CONFIGS["c1"])
    spec.pop("depth")
    raw, _, par = F.generate(**spec)
    edges = [(int(p), c) for c in range(par.shape[0]) for p in par[c] if p >= 0]
    with open(os.path.join(HERE, "c1_dag"), "w") as f:
        for p, c in edges:
            f.write("%d %d\n" % (p, c))
    tmp = tempfile.mkdtemp()
    try:
        csv = os.path.join(tmp, "c1.csv")
        F.write_csv(csv, raw)
        import subprocess
        subprocess.check_call([O.REF_DRIVER, "mle", csv, "1", os.path.join(HERE, "c1_dag"), os.path.join(tmp, "o"),
                               os.path.join(HERE, "c1_param_alpha1")], stdout=subprocess.DEVNULL)
        subprocess.check_call([O.REF_DRIVER, "bnl", csv, "0.05", os.path.join(tmp, "bnl")], stdout=subprocess.DEVNULL)
        shutil.copyfile(os.path.join(tmp, "bnl_param"), os.path.join(HERE, "c1_bnl_param"))
        assert open(os.path.join(tmp, "bnl_struct")).read() == open(os.path.join(HERE, "c1_struct")).read()
    finally:
        shutil.rmtree(tmp)


def main():
    O.build()
    assert O.ref_available(), "reference-built driver missing"
    mle_golden()
    if "--mle-only" in sys.argv:
        return
    rng = np.random.default_rng(1234)
    # alarm
    alarm_csv = os.path.join(REF, "dataset/alarm/alarm_s5000")
    names, cols, card = O.read_csv_columns(alarm_csv)
    np.savez_compressed(os.path.join(HERE, "alarm_s5000.npz"), cols=cols, card=card, names=np.array(names))
    shutil.copyfile(os.path.join(REF, "dataset/alarm/alarm_s5000_struct"), os.path.join(HERE, "alarm_s5000_struct"))
    tmp = tempfile.mkdtemp()
    r = O.ref_pc(alarm_csv, os.path.join(tmp, "alarm"))
    shutil.copyfile(os.path.join(tmp, "alarm_sepsets"), os.path.join(HERE, "alarm_sepsets"))
    assert open(os.path.join(tmp, "alarm_struct")).read() == open(os.path.join(HERE, "alarm_s5000_struct")).read()
    ref_tests(alarm_csv, sample_tests(cols.shape[0], card, rng, 400, 4), os.path.join(HERE, "alarm_tests.txt"))
    # seeded synthetic configs
    for name in ("c1", "c2"):
        raw, depth, spec = F.make_config(name)
        csv = os.path.join(tmp, name + ".csv")
        F.write_csv(csv, raw)
        rr = O.ref_pc(csv, os.path.join(tmp, name), threads=1, depth=depth)  # T>1 races on sepset
        for suf in ("_struct", "_sepsets"):
            shutil.copyfile(os.path.join(tmp, name + suf), os.path.join(HERE, name + suf))
        meta = {"sha256": hashlib.sha256(raw.tobytes()).hexdigest(), "shape": list(raw.shape), "depth": depth,
                "spec": spec, "ref_num_ci_test_1_thread": rr["num_ci_test"]}
        with open(os.path.join(HERE, name + "_meta.json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        if name == "c1":
            cl, cd = O.relabel(raw)
            ref_tests(csv, sample_tests(raw.shape[0], cd, rng, 400, 5), os.path.join(HERE, "c1_tests.txt"))
    shutil.rmtree(tmp)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
