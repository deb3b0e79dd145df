"""Full-size skeleton parity on the benchmark workloads c3, c4 and c5.

c3: 223 nodes x 500,000 samples, depth 5; c4: 1,041 nodes x 100,000 samples with up to 21
states (the spec workload); c5: 64 independent datasets of 20-200 nodes and 1,000 to
200,000 samples learned in one engine.  The fixtures (tests/golden/full_<cfg>.json, written
by tests/golden/make_full.py) hold the oracle's result at these sizes as digests: sha256 of
the generated data, per-level deterministic test counts and surviving edges, and sha256 of
the adjacency and of the sorted separating sets.  The oracle is pinned to the reference's
own PC-stable code on alarm, c1 and c2 (test_oracle.py).  Every digest must match exactly.
"""
import json
import os

import pytest

from conftest import GOLDEN
from oracle import oracle as O
import fastpgm_gb300 as F
from fastpgm_gb300 import configs as C

pytestmark = pytest.mark.gpu


def fixture(name):
    with open(os.path.join(GOLDEN, "full_%s.json" % name)) as f:
        return json.load(f)


def check_job(got_adj, got_seps, job):
    d = O.skeleton_digest(got_adj, got_seps)
    assert d["n_removed"] == job["n_removed"], "removed edges differ"
    assert d["adj_sha256"] == job["adj_sha256"], "skeleton differs"
    assert d["sep_sha256"] == job["sep_sha256"], "separating sets differ"


@pytest.mark.parametrize("name", ["c3", "c4"])
def test_full_size_skeleton_matches_oracle(name):
    fx = fixture(name)
    raw, depth, _ = C.make_config(name)
    job = fx["jobs"][0]
    assert O.sha256(raw) == job["sha256"], "the seeded sampler produced other data on this host"
    assert depth == fx["depth"]
    with F.Engine(0) as e:
        e.upload(raw)
        st = e.pc_skeleton(depth=depth).to_dict()
        res = e.result()
    assert st["tests"] == job["tests"], "per-level CI test counts differ"
    assert st["edges_after"] == job["edges_after"], "per-level edge counts differ"
    check_job(res["adj"], res["sepsets"], job)


def test_full_size_64_jobs_match_oracle():
    """All 64 datasets of c5 at full size in one engine: every job's skeleton and separating
    sets equal the oracle's run of that dataset alone, and each level's test count equals the
    sum of the jobs' counts at that level.  (A job whose oracle run is missing from the
    fixture -- the oracle needs hours for the largest -- is skipped, and then the level sums
    too; at most one.)"""
    fx = fixture("c5")
    data, depth = C.make_jobs(C.c5_jobs())
    assert len(data) == len(fx["jobs"]) == 64
    for raw, job in zip(data, fx["jobs"]):
        if job is not None:
            assert O.sha256(raw) == job["sha256"], "the seeded sampler produced other data on this host"
    with F.Engine(0) as e:
        e.upload_jobs(data)
        st = e.pc_skeleton(depth=depth).to_dict()
        res = e.result()
        offsets = e.job_offsets
    if fx["level_tests"] is not None:  # every job's oracle run is in the fixture
        assert st["tests"] == fx["level_tests"], "per-level CI test counts differ"
    checked = 0
    for (adj, seps), job in zip(F.split_jobs(res, offsets), fx["jobs"]):
        if job is not None:
            check_job(adj, seps, job)
            checked += 1
    assert checked >= 63
