"""Offline sweep of the tier-2 method, keyed by (samples, |Z|, joint cardinality).

A CI test whose joint table is too large for shared memory and whose Z strata overflow the
compact kernel's shared hash is counted one of two ways: the compact kernel's global strata
hash, or the partition kernel (samples split by stratum into shared-memory partitions).  The
engine chooses per test with its online autotuner (ci_kernels.cuh, tier2_pick_partitions):
per (samples, |Z|, cells/samples) bucket it times both methods on the tests it runs and
prefers the faster.  This script is the offline alternative: it times both methods on
batches of random tests over synthetic datasets of every sample-count bucket and writes a
fixed table, which an engine uses instead when FPGM_TUNE_TABLE names it.  (Measured on
GB300, such a table lost 4% at the 1,041-node workload against the fixed cut-over: random
batches are not the tests a skeleton runs, which is why the online tuner is the default.)

Run on a GPU:  python -m fastpgm_gb300.tune --out PATH [--quick]
"""
import argparse
import datetime
import math
import os
import time

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(PKG, "tune_table.txt")  # default output path (not loaded unless FPGM_TUNE_TABLE names it)

KTUNE_SB, KTUNE_DB, KTUNE_CB = 6, 12, 6   # the engine's kTuneSB / kTuneDB / kTuneCB
SAMPLES = [10000, 20000, 40000, 80000, 160000, 240000]  # one per sample bucket
CARDS = [(2, 5), (3, 9), (6, 12), (2, 21)]


def tune_index(S, d, cells):
    """The engine's tune_index(): (sample bucket, |Z| bucket, cells/samples bucket)."""
    sb, lim = 0, 12500
    while sb < KTUNE_SB - 1 and S >= lim:
        sb += 1
        lim *= 2
    db = 0 if d < 1 else min(d, KTUNE_DB) - 1
    r = cells / max(S, 1)
    cb, lim = 0, 4.0
    while cb < KTUNE_CB - 1 and r >= lim:
        cb += 1
        lim *= 4.0
    return sb, db, cb


def _engine(cutover):
    import fastpgm_gb300 as F
    saved = {k: os.environ.get(k) for k in ("FPGM_PART_CUTOVER", "FPGM_WIDE", "FPGM_TUNE_TABLE")}
    os.environ["FPGM_PART_CUTOVER"] = str(cutover)
    os.environ["FPGM_WIDE"] = "0"      # the method alone, without the tail-wave spreading
    os.environ["FPGM_TUNE_TABLE"] = "off"
    try:
        return F.Engine(0)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _time(eng, tests, d, reps):
    best = math.inf
    for _ in range(reps):
        t0 = time.perf_counter()
        eng.ci_test_batch(tests, d)
        best = min(best, time.perf_counter() - t0)
    return best


def sweep(out=TABLE, quick=False, log=print):
    import fastpgm_gb300 as F
    part, hashed = _engine(0), _engine(1 << 62)
    n_vars, batch = 16, 608
    samples = SAMPLES[2:4] if quick else SAMPLES
    ds = range(4, 9) if quick else range(2, 13)
    votes = {}
    try:
        for S in samples:
            for ci, card in enumerate(CARDS):
                raw, _, _ = F.generate(n_nodes=n_vars, n_samples=S, seed=7000 + 10 * ci + S % 7, avg_indegree=2.0,
                                       max_indegree=4, card=card, dirichlet=0.5)
                cd = part.upload(raw)
                hashed.upload(raw)
                rng = np.random.default_rng(S + ci)
                for d in ds:
                    if 2 + d > n_vars:
                        continue
                    tests = np.array([rng.choice(n_vars, size=2 + d, replace=False) for _ in range(batch)],
                                     dtype=np.int32)
                    cells = np.array([float(np.prod(cd[t].astype(np.float64))) for t in tests])
                    keys = [tune_index(S, d, c) for c in cells]
                    for key in sorted(set(keys)):
                        sel = tests[[k == key for k in keys]]
                        if len(sel) < 64:
                            continue
                        part.ci_test_batch(sel[:8], d)  # warm-up
                        tp = _time(part, sel, d, 2)
                        th = _time(hashed, sel, d, 2)
                        v = votes.setdefault(key, [0.0, 0.0])
                        v[0] += tp
                        v[1] += th
                        log("S=%d card=%s d=%d bucket=%s tests=%d partition %.2f ms, global hash %.2f ms"
                            % (S, card, d, key, len(sel), tp * 1e3, th * 1e3))
    finally:
        part.close()
        hashed.close()
    with open(out, "w") as f:
        f.write("# Tier-2 method per (sample bucket, |Z| bucket, cells/samples bucket): 1 partition kernel, "
                "0 global strata hash\n")
        f.write("# written by: python -m fastpgm_gb300.tune (%s)\n" % datetime.date.today().isoformat())
        f.write("# columns: sb db cb method  partition_ms global_hash_ms\n")
        for key in sorted(votes):
            tp, th = votes[key]
            f.write("%d %d %d %d  %.3f %.3f\n" % (key[0], key[1], key[2], 1 if tp < th else 0, tp * 1e3, th * 1e3))
    return votes


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--quick", action="store_true")
    a = ap.parse_args()
    sweep(a.out, a.quick)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
