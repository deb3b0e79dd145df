"""Seeded synthetic workloads with the shapes of the PC-stable benchmark configurations.

c1  37 nodes, 46 edges, max in-degree 4, cardinality U{2,3,4}, Dirichlet(1), 5,000 samples
    (the Alarm network's shape; the reference also ships the real alarm_s5000)
c2  100 nodes, average in-degree 2 (max 5), cardinality U{2..5}, Dirichlet(0.5), 50,000 samples
c3  223 nodes, average in-degree 1.5, cardinality 3, Dirichlet(1), 500,000 samples, |Z| <= 4 (depth 5)
c4  1,041 nodes (Munin3's size), average in-degree 1.3 (max 3), cardinality U{2..8} with a 20% tail
    U{9..21}, Dirichlet(0.3), 100,000 samples
c5  64 independent jobs: nodes U[20,200], samples log-uniform [1e3, 2e5], cardinality U{2..6},
    average in-degree U[1.5,2.5] (max 5), Dirichlet(1)

All data are synthetic: random DAG + Dirichlet CPTs + forward sampling from a fixed seed
(fpgm_generate_network), identical on x86-64 and AArch64.
"""
import numpy as np

CONFIGS = {
    "c1": dict(n_nodes=37, n_edges=46, max_indegree=4, card=(2, 4), dirichlet=1.0, n_samples=5000, seed=1,
               depth=1000),
    "c2": dict(n_nodes=100, avg_indegree=2.0, max_indegree=5, card=(2, 5), dirichlet=0.5, n_samples=50000, seed=2,
               depth=1000),
    "c3": dict(n_nodes=223, avg_indegree=1.5, max_indegree=4, card=(3, 3), dirichlet=1.0, n_samples=500000, seed=3,
               depth=5),
    "c4": dict(n_nodes=1041, avg_indegree=1.3, max_indegree=3, card=(2, 8), tail=(0.2, 9, 21), dirichlet=0.3,
               n_samples=100000, seed=4, depth=1000),
}


def c5_jobs(seed=5, n_jobs=64):
    """Parameters of the 64 independent structure-learning jobs of c5."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        n = int(rng.integers(20, 201))
        S = int(round(10 ** rng.uniform(3.0, np.log10(2e5))))
        jobs.append(dict(n_nodes=n, avg_indegree=float(rng.uniform(1.5, 2.5)), max_indegree=5, card=(2, 6),
                         dirichlet=1.0, n_samples=S, seed=1000 + j, depth=1000))
    return jobs


def make_jobs(jobs, generate=None):
    """Generate the datasets of a list of job parameter dicts (c5_jobs()).  Returns
    (list of raw uint8 [n_j, S_j], depth).  generate: the sampler to call (default the
    engine library's; any function with fastpgm_gb300.generate's signature and output)."""
    if generate is None:
        from . import generate
    out, depth = [], 1000
    for spec in jobs:
        spec = dict(spec)
        depth = spec.pop("depth")
        cols, card, par = generate(**spec)
        out.append(cols)
    return out, depth


def split_jobs(result, offsets):
    """Per-dataset views of a multi-dataset skeleton result (Engine.result() with the
    engine's job_offsets): [(adj [n_j, n_j], sepsets {(a, b): z} in local numbering)]."""
    out = []
    for j in range(len(offsets) - 1):
        lo, hi = int(offsets[j]), int(offsets[j + 1])
        adj = result["adj"][lo:hi, lo:hi]
        seps = {(a - lo, b - lo): tuple(v - lo for v in z) for (a, b), z in result["sepsets"].items()
                if lo <= a < hi}
        out.append((adj, seps))
    return out


def make_config(name, n_samples=None, n_nodes=None, generate=None):
    """Generate a config's data.  Returns (columns raw uint8 [n,S], depth, spec dict).
    generate: the sampler to call (default the engine library's)."""
    if generate is None:
        from . import generate
    spec = dict(CONFIGS[name])
    if n_samples is not None:
        spec["n_samples"] = n_samples
    if n_nodes is not None:
        spec["n_nodes"] = n_nodes
    depth = spec.pop("depth")
    cols, card, par = generate(**spec)
    return cols, depth, spec
