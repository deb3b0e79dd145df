"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm
import this module, and only as the checker.  It wraps
``oracle/_build/liboracle.so`` (the plain-C restatement in ``pc_oracle.c``)
and, where the reference tree exists, the reference-built
``oracle/_ref/ref_driver``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
DATAGEN_PATH = os.path.join(HERE, "_build", "libdatagen.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")
# The FastPGM source tree the reference-built driver compiles from (only where it exists).
REFERENCE_TREE = os.environ.get("FASTPGM_REFERENCE", "/root/reference")


class CIResult(ctypes.Structure):
    _fields_ = [("table_hash", ctypes.c_uint64), ("cell_hash", ctypes.c_uint64), ("cells", ctypes.c_int64),
                ("df", ctypes.c_int32),
                ("g2", ctypes.c_double), ("p_value", ctypes.c_double), ("independent", ctypes.c_int32)]


class PCStats(ctypes.Structure):
    _fields_ = [("n_levels", ctypes.c_int32), ("tests", ctypes.c_int64 * 64),
                ("edges_after", ctypes.c_int32 * 64), ("seconds", ctypes.c_double * 64)]


def build(quiet=True):
    """Compile the C restatement (and the reference-built driver when the tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "oracle"], stdout=out)
    if os.path.isdir(REFERENCE_TREE):
        subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + REFERENCE_TREE], stdout=out)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.oracle_relabel.argtypes = [u8p, ctypes.c_int, ctypes.c_int64, u8p, u8p]
        L.oracle_relabel.restype = None
        L.oracle_ci_tests.argtypes = [u8p, u8p, ctypes.c_int, ctypes.c_int64, i32p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_int, ctypes.POINTER(CIResult)]
        L.oracle_ci_tests.restype = ctypes.c_int
        L.oracle_pc_skeleton.argtypes = [u8p, u8p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, u8p, i32p, i32p, ctypes.POINTER(PCStats)]
        L.oracle_pc_skeleton.restype = ctypes.c_int
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.oracle_mle_cpts.argtypes = [u8p, u8p, ctypes.c_int, ctypes.c_int64, i32p, i32p, ctypes.c_int, i64p,
                                      ctypes.POINTER(ctypes.c_double)]
        L.oracle_mle_cpts.restype = ctypes.c_int
        _lib = L
    return _lib


_gen = None


class GenSpec(ctypes.Structure):
    """fpgm_gen_spec of the engine's C header (same field order and types)."""
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_edges", ctypes.c_int32), ("avg_indegree", ctypes.c_double),
                ("max_indegree", ctypes.c_int32), ("card_min", ctypes.c_int32), ("card_max", ctypes.c_int32),
                ("tail_frac", ctypes.c_double), ("tail_min", ctypes.c_int32), ("tail_max", ctypes.c_int32),
                ("dirichlet_alpha", ctypes.c_double), ("n_samples", ctypes.c_int64), ("seed", ctypes.c_uint64)]


def generate(n_nodes, n_samples, seed, n_edges=0, avg_indegree=2.0, max_indegree=4, card=(2, 4),
             tail=(0.0, 2, 2), dirichlet=1.0):
    """The seeded network sampler built on its own (_build/libdatagen.so), for the CPU arms:
    same arguments and bytes as fastpgm_gb300.generate, without loading the engine library.
    Returns (columns uint8 [n, S] raw ids, card, parents)."""
    global _gen
    if _gen is None:
        if not os.path.exists(DATAGEN_PATH):
            build()
        _gen = ctypes.CDLL(DATAGEN_PATH)
        _gen.fpgm_generate_network.argtypes = [ctypes.POINTER(GenSpec), ctypes.POINTER(ctypes.c_uint8),
                                               ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32)]
        _gen.fpgm_generate_network.restype = ctypes.c_int
    spec = GenSpec(n_nodes, n_edges, avg_indegree, max_indegree, card[0], card[1], tail[0], tail[1], tail[2],
                   dirichlet, n_samples, seed)
    cols = np.empty((n_nodes, n_samples), dtype=np.uint8)
    c = np.empty(n_nodes, dtype=np.uint8)
    par = np.full((n_nodes, max(1, max_indegree)), -1, dtype=np.int32)
    rc = _gen.fpgm_generate_network(ctypes.byref(spec), _u8(cols), _u8(c), _i32(par))
    if rc != 0:
        raise RuntimeError("fpgm_generate_network failed: %d" % rc)
    return cols, c, par


def _u8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _i32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def relabel(raw):
    """First-appearance ids per column; raw is [n_vars, n_samples] uint8.  Returns (cols, card)."""
    raw = np.ascontiguousarray(raw, dtype=np.uint8)
    n, S = raw.shape
    out = np.empty_like(raw)
    card = np.empty(n, dtype=np.uint8)
    lib().oracle_relabel(_u8(raw), n, S, _u8(out), _u8(card))
    return out, card


def ci_tests(cols, card, tests, d, alpha=0.05, threads=8):
    """Run CI tests given as an int32 array [n_tests, 2+d] of (x, y, z1..zd)."""
    cols = np.ascontiguousarray(cols, dtype=np.uint8)
    card = np.ascontiguousarray(card, dtype=np.uint8)
    tests = np.ascontiguousarray(tests, dtype=np.int32).reshape(-1, 2 + d)
    res = (CIResult * max(1, len(tests)))()
    rc = lib().oracle_ci_tests(_u8(cols), _u8(card), cols.shape[0], cols.shape[1], _i32(tests), len(tests), d,
                               alpha, threads, res)
    if rc != 0:
        raise RuntimeError("oracle_ci_tests failed: %d" % rc)
    return [res[i] for i in range(len(tests))]


def pc_skeleton(cols, card, alpha=0.05, depth=1000, threads=8, max_z=32):
    """Returns dict(adj [n,n] uint8, sepsets {(a,b): tuple}, stats)."""
    cols = np.ascontiguousarray(cols, dtype=np.uint8)
    card = np.ascontiguousarray(card, dtype=np.uint8)
    n, S = cols.shape
    E = n * (n - 1) // 2
    adj = np.zeros((n, n), dtype=np.uint8)
    sep_len = np.zeros(E, dtype=np.int32)
    sep_vars = np.zeros(E * max_z, dtype=np.int32)
    st = PCStats()
    rc = lib().oracle_pc_skeleton(_u8(cols), _u8(card), n, S, alpha, depth, threads, max_z, _u8(adj),
                                  _i32(sep_len), _i32(sep_vars), ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("oracle_pc_skeleton failed: %d" % rc)
    iu, ju = np.triu_indices(n, 1)
    seps = {}
    for e in np.nonzero(sep_len >= 0)[0]:
        L = int(sep_len[e])
        seps[(int(iu[e]), int(ju[e]))] = tuple(int(v) for v in sep_vars[e * max_z:e * max_z + L])
    stats = {"n_levels": st.n_levels,
             "tests": [int(st.tests[i]) for i in range(st.n_levels)],
             "edges_after": [int(st.edges_after[i]) for i in range(st.n_levels)],
             "seconds": [float(st.seconds[i]) for i in range(st.n_levels)]}
    return {"adj": adj, "sepsets": seps, "stats": stats}


def sha256(a):
    """sha256 hex digest of an array's bytes (C order)."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def skeleton_digest(adj, sepsets):
    """Compact, order-free fingerprint of a skeleton result: sha256 of the upper triangle
    of the 0/1 adjacency (row-major) and of the sorted separating-set lines "a b:z1 z2 ..."."""
    import hashlib
    adj = np.asarray(adj, dtype=np.uint8)
    iu = np.triu_indices(adj.shape[0], 1)
    lines = "".join("%d %d:%s\n" % (a, b, " ".join(map(str, z))) for (a, b), z in sorted(sepsets.items()))
    return {"adj_sha256": sha256((adj[iu] != 0).astype(np.uint8)),
            "sep_sha256": hashlib.sha256(lines.encode()).hexdigest(), "n_removed": len(sepsets)}


def read_csv_columns(path):
    """Load a CSV the way Dataset::LoadCSVTrainingData(path, str_val=true) does: header = names,
    every cell a string, ids by first appearance per column.  Returns (names, cols, card)."""
    with open(path) as f:
        header = f.readline().rstrip().split(",")
        rows = [line.rstrip().split(",") for line in f if line.strip()]
    n, S = len(header), len(rows)
    cols = np.empty((n, S), dtype=np.uint8)
    card = np.empty(n, dtype=np.uint8)
    for v in range(n):
        ids = {}
        for s in range(S):
            cols[v, s] = ids.setdefault(rows[s][v], len(ids))
        card[v] = len(ids)
    return header, cols, card


def ref_available():
    return os.path.exists(REF_DRIVER)


def ref_pc(csv_path, out_prefix, alpha=0.05, threads=1, group_size=1, depth=1000, verbose=0):
    """Run the reference-built driver: writes <out_prefix>_struct and _sepsets."""
    out = subprocess.run([REF_DRIVER, "pc", csv_path, repr(alpha), str(threads), str(group_size), str(depth),
                          out_prefix, str(verbose)], check=True, capture_output=True, text=True).stdout
    line = [l for l in out.splitlines() if l.startswith("ref_pc_seconds")][-1].split()
    return {"seconds": float(line[1]), "num_ci_test": int(line[3]), "stdout": out}


def read_sepsets(path):
    seps = {}
    with open(path) as f:
        for line in f:
            a, rest = line.split(":")
            i, j = a.split()
            seps[(int(i), int(j))] = tuple(int(v) for v in rest.split())
    return seps


def parent_csr(parents):
    """Parent lists (any iterables; duplicates and order ignored, as in the reference's
    parent set) -> (offsets int32 [n+1], sorted parents int32)."""
    off = [0]
    flat = []
    for p in parents:
        q = sorted(set(int(x) for x in p if int(x) >= 0))
        flat += q
        off.append(len(flat))
    return np.array(off, dtype=np.int32), np.array(flat if flat else [0], dtype=np.int32)


def mle_cpts(cols, card, parents, alpha=1):
    """Maximum-likelihood tables with Laplace smoothing alpha for a known DAG (relabelled
    columns).  Returns a list of float64 arrays, node v's over (v, sorted parents), v slowest."""
    cols = np.ascontiguousarray(cols, dtype=np.uint8)
    card = np.ascontiguousarray(card, dtype=np.uint8)
    n, S = cols.shape
    off, flat = parent_csr(parents)
    toff = np.zeros(n + 1, dtype=np.int64)
    i64p = ctypes.POINTER(ctypes.c_int64)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib().oracle_mle_cpts(_u8(cols), _u8(card), n, S, _i32(off), _i32(flat), int(alpha),
                               toff.ctypes.data_as(i64p), None)
    if rc != 0:
        raise RuntimeError("oracle_mle_cpts: table too large")
    pot = np.zeros(int(toff[-1]), dtype=np.float64)
    lib().oracle_mle_cpts(_u8(cols), _u8(card), n, S, _i32(off), _i32(flat), int(alpha), toff.ctypes.data_as(i64p),
                          pot.ctypes.data_as(dp))
    return [pot[toff[v]:toff[v + 1]] for v in range(n)]


def ref_mle(csv, alpha, edges, workdir):
    """The reference's own ParameterLearning on csv for the directed edges [(parent, child)]
    (oracle/_ref/ref_driver mle).  Returns {node: (related variables, potentials)}."""
    ein = os.path.join(workdir, "mle_edges")
    out = os.path.join(workdir, "mle_out")
    with open(ein, "w") as f:
        for p, c in edges:
            f.write("%d %d\n" % (p, c))
    subprocess.run([REF_DRIVER, "mle", csv, str(int(alpha)), ein, out], check=True, capture_output=True)
    res = {}
    for line in open(out):
        head, pots = line.split(":")
        h = [int(x) for x in head.split()]
        res[h[0]] = (h[2:2 + h[1]], np.array([float(x) for x in pots.split()]))
    return res
