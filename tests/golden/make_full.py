"""Full-size skeleton fixtures for the c3, c4 and c5 workloads, from the CPU oracle.

The reference's own code cannot run these sizes here: its dense per-test tables
(Counts3D, dz*dx*dy cells) at c4's deep levels need more memory than any host has, and
single-threaded (the only race-free setting for its separating sets) c3 or c5 would take
hours.  The fixtures therefore come from the plain-C restatement (oracle/pc_oracle.c),
which the other fixtures pin to the reference on alarm, c1 and c2 (sepsets, CPDAGs,
per-level test counts, 800 per-test vectors).

Writes tests/golden/full_<cfg>.json with, per dataset (c5: per job):
  sha256        of the raw generated columns (the sampler's bytes must match on the test host)
  tests         deterministic CI tests per level (sequential group-size-1 count)
  edges_after   skeleton edges left after each level
  adj_sha256    of the upper triangle of the 0/1 adjacency, row-major
  sep_sha256    of the sorted separating-set lines "a b:z1 z2 ...\\n" (a < b)
  n_removed     removed edges (one separating set each)
and, for c5, the level totals over all jobs (what a multi-dataset skeleton reports).

Run:  python tests/golden/make_full.py [c3] [c4] [c5] [--workers N] [--partial]   (default: all
three; c5 takes longest: its 64 jobs run N at a time in separate processes, each job's digest
cached under tests/golden/.full_cache/; jobs already in full_c5.json are kept and only the
missing ones run; --partial writes c5 from the fixture and the cached jobs alone, a missing
job as null, which the GPU test then skips)
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fastpgm_gb300 import configs as C  # noqa: E402  (pure Python: parameters only)
from oracle import oracle as O  # noqa: E402


def dataset_digest(raw, depth, threads):
    cols, card = O.relabel(raw)
    t0 = time.perf_counter()
    r = O.pc_skeleton(cols, card, depth=depth, threads=threads)
    dt = time.perf_counter() - t0
    d = O.skeleton_digest(r["adj"], r["sepsets"])
    d.update({"sha256": O.sha256(raw), "shape": list(raw.shape), "tests": r["stats"]["tests"],
              "edges_after": r["stats"]["edges_after"]})
    return d, dt


CACHE = os.path.join(HERE, ".full_cache")


def _c5_job(args):
    """One c5 job's digest in a worker process (cached by job index)."""
    j, threads = args
    path = os.path.join(CACHE, "c5_job%02d.json" % j)
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    spec = dict(C.c5_jobs()[j])
    depth = spec.pop("depth")
    raw, _, _ = O.generate(**spec)
    d, dt = dataset_digest(raw, depth, threads)
    os.makedirs(CACHE, exist_ok=True)
    with open(path + ".tmp", "w") as f:
        json.dump(d, f)
    os.replace(path + ".tmp", path)
    print("c5 job %d: %d x %d, %d tests, %.1f s" % (j, raw.shape[0], raw.shape[1], sum(d["tests"]), dt), flush=True)
    return d


def main():
    names = [a for a in sys.argv[1:] if a in ("c3", "c4", "c5")] or ["c3", "c4", "c5"]
    workers = int(sys.argv[sys.argv.index("--workers") + 1]) if "--workers" in sys.argv else 1
    threads = max(1, (os.cpu_count() or 1) // workers)
    O.build()
    for name in names:
        t0 = time.perf_counter()
        if name == "c5":
            import multiprocessing as mp
            specs = C.c5_jobs()
            depth = specs[0]["depth"]
            # largest first, so the long jobs start at once
            order = sorted(range(len(specs)), key=lambda j: -specs[j]["n_samples"] * specs[j]["n_nodes"])
            done = {}
            fixture = os.path.join(HERE, "full_c5.json")
            if os.path.exists(fixture):  # jobs already in the fixture are kept
                with open(fixture) as f:
                    old = json.load(f)
                if len(old.get("jobs", [])) == len(specs):
                    done = {j: d for j, d in enumerate(old["jobs"]) if d is not None}
            for j in order:
                path = os.path.join(CACHE, "c5_job%02d.json" % j)
                if j not in done and os.path.exists(path):
                    with open(path) as f:
                        done[j] = json.load(f)
            todo = [j for j in order if j not in done]
            if todo and "--partial" not in sys.argv:  # --partial: a missing job stays null
                with mp.get_context("spawn").Pool(min(workers, len(todo))) as pool:
                    done.update(zip(todo, pool.map(_c5_job, [(j, threads) for j in todo], chunksize=1)))
            jobs = [done.get(j) for j in range(len(specs))]
            have = [d for d in jobs if d is not None]
            L = max(len(d["tests"]) for d in have)
            out = {"config": name, "depth": depth, "jobs": jobs,
                   "level_tests": ([sum(d["tests"][i] for d in have if i < len(d["tests"])) for i in range(L)]
                                   if len(have) == len(jobs) else None)}
        else:
            raw, depth, spec = C.make_config(name, generate=O.generate)
            d, dt = dataset_digest(raw, depth, threads)
            out = {"config": name, "depth": depth, "spec": spec, "jobs": [d]}
        out["oracle_seconds"] = round(time.perf_counter() - t0, 1)
        out["oracle_threads"] = threads
        with open(os.path.join(HERE, "full_%s.json" % name), "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)
        print("%s: %.1f s" % (name, out["oracle_seconds"]), flush=True)


if __name__ == "__main__":
    main()
