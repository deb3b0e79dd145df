"""GB300 PC-stable CI-testing engine -- Python front end over the C ABI.

The compute lives in ``lib/libfastpgm_gb300.so`` (hand-written sm_103a CUDA
kernels + C++ host code); this module only marshals arrays through ctypes.
There is no CPU fallback: if the library is missing or no GPU is visible,
the calls that need one raise.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libfastpgm_gb300.so")
CLI_PATH = os.path.join(PKG, "bin", "fastpgm")

FPGM_OK = 0
FPGM_ERR_INVALID, FPGM_ERR_OOM, FPGM_ERR_CUDA, FPGM_ERR_TIMEOUT, FPGM_ERR_IO, FPGM_ERR_UNSUPPORTED, FPGM_ERR_STATE = (
    -1, -2, -3, -4, -5, -6, -7)
FPGM_MODE_BATCHED = 0
FPGM_MODE_PLAIN = 1
MAX_COND = 30

EXPORTED = ["fpgm_last_error", "fpgm_engine_create", "fpgm_engine_destroy", "fpgm_dataset_upload",
            "fpgm_dataset_upload_jobs", "fpgm_mle_cpts", "fpgm_shd_bif", "fpgm_bnl_pcstable",
            "fpgm_dataset_download", "fpgm_ci_test", "fpgm_ci_test_batch", "fpgm_pc_skeleton",
            "fpgm_pc_result_sizes", "fpgm_pc_result_fetch", "fpgm_orient_cpdag", "fpgm_write_struct",
            "fpgm_bnsl_pcstable", "fpgm_generate_network", "fpgm_write_csv", "fpgm_ci_test_noalloc"]


class CIResult(ctypes.Structure):
    _fields_ = [("table_hash", ctypes.c_uint64), ("cell_hash", ctypes.c_uint64), ("cells", ctypes.c_int64),
                ("df", ctypes.c_int32),
                ("independent", ctypes.c_int32), ("g2", ctypes.c_double), ("p_value", ctypes.c_double),
                ("rechecked", ctypes.c_int32), ("path", ctypes.c_int32)]


class PCStats(ctypes.Structure):
    _fields_ = [("n_levels", ctypes.c_int32), ("tests", ctypes.c_int64 * 64),
                ("tests_executed", ctypes.c_int64 * 64), ("edges_after", ctypes.c_int32 * 64),
                ("waves", ctypes.c_int32 * 64), ("ms", ctypes.c_double * 64), ("rechecks", ctypes.c_int64),
                ("near_ties", ctypes.c_int64), ("large_tests", ctypes.c_int64), ("max_abs_dp", ctypes.c_double),
                ("count_ms", ctypes.c_double), ("count_bytes", ctypes.c_double), ("large_ms", ctypes.c_double),
                ("count_launches", ctypes.c_int64), ("kernel_launches", ctypes.c_int64), ("span_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("large_bytes", ctypes.c_double), ("gram_ms", ctypes.c_double),
                ("gram_flops", ctypes.c_double), ("gram_tests", ctypes.c_int64), ("tune_buckets", ctypes.c_int32),
                ("tune_partition", ctypes.c_int32), ("tune_timed", ctypes.c_int64), ("graph_ms", ctypes.c_double)]

    def to_dict(self):
        L = self.n_levels
        return {"n_levels": L, "tests": [int(self.tests[i]) for i in range(L)],
                "tests_executed": [int(self.tests_executed[i]) for i in range(L)],
                "edges_after": [int(self.edges_after[i]) for i in range(L)],
                "waves": [int(self.waves[i]) for i in range(L)], "ms": [float(self.ms[i]) for i in range(L)],
                "rechecks": int(self.rechecks), "near_ties": int(self.near_ties),
                "large_tests": int(self.large_tests), "max_abs_dp": float(self.max_abs_dp),
                "count_ms": float(self.count_ms), "count_bytes": float(self.count_bytes),
                "large_ms": float(self.large_ms),
                "count_launches": int(self.count_launches), "kernel_launches": int(self.kernel_launches),
                "span_ms": float(self.span_ms), "total_ms": float(self.total_ms),
                "large_bytes": float(self.large_bytes), "gram_ms": float(self.gram_ms),
                "gram_flops": float(self.gram_flops), "gram_tests": int(self.gram_tests),
                "tune_buckets": int(self.tune_buckets), "tune_partition": int(self.tune_partition),
                "tune_timed": int(self.tune_timed), "graph_ms": float(self.graph_ms)}


class GenSpec(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_edges", ctypes.c_int32), ("avg_indegree", ctypes.c_double),
                ("max_indegree", ctypes.c_int32), ("card_min", ctypes.c_int32), ("card_max", ctypes.c_int32),
                ("tail_frac", ctypes.c_double), ("tail_min", ctypes.c_int32), ("tail_max", ctypes.c_int32),
                ("dirichlet_alpha", ctypes.c_double), ("n_samples", ctypes.c_int64), ("seed", ctypes.c_uint64)]


class FpgmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("fastpgm_gb300 error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load():
    """Load the engine library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    u8p, i32p, vp = ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p
    L.fpgm_last_error.restype = ctypes.c_char_p
    L.fpgm_engine_create.argtypes = [ctypes.c_int32, ctypes.POINTER(vp)]
    L.fpgm_engine_destroy.argtypes = [vp]
    L.fpgm_dataset_upload.argtypes = [vp, u8p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, u8p]
    L.fpgm_bnl_pcstable.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_char_p,
                                    ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32]
    L.fpgm_shd_bif.argtypes = [ctypes.c_char_p, ctypes.c_int32, i32p, ctypes.c_int32, i32p]
    L.fpgm_mle_cpts.argtypes = [vp, i32p, i32p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_double)]
    L.fpgm_dataset_upload_jobs.argtypes = [vp, ctypes.c_int32, i32p, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, u8p]
    L.fpgm_dataset_download.argtypes = [vp, u8p]
    L.fpgm_ci_test.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, i32p, ctypes.c_int32, ctypes.c_double,
                               ctypes.c_int32, ctypes.POINTER(CIResult)]
    L.fpgm_ci_test_batch.argtypes = [vp, i32p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                     ctypes.POINTER(CIResult)]
    L.fpgm_pc_skeleton.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(PCStats)]
    L.fpgm_pc_result_sizes.argtypes = [vp, i32p, i32p, ctypes.POINTER(ctypes.c_int64)]
    L.fpgm_pc_result_fetch.argtypes = [vp, u8p, i32p, i32p, i32p]
    L.fpgm_orient_cpdag.argtypes = [ctypes.c_int32, u8p, ctypes.c_int32, i32p, i32p, i32p, i32p, i32p]
    L.fpgm_write_struct.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p), i32p,
                                    ctypes.c_int32, ctypes.c_int32]
    L.fpgm_bnsl_pcstable.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                     ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    L.fpgm_generate_network.argtypes = [ctypes.POINTER(GenSpec), u8p, u8p, i32p]
    L.fpgm_write_csv.argtypes = [ctypes.c_char_p, u8p, ctypes.c_int32, ctypes.c_int64, ctypes.c_char_p]
    L.fpgm_ci_test_noalloc.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                       ctypes.c_int32, i32p, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, vp, vp]
    for name in EXPORTED:
        if name != "fpgm_last_error":
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _check(rc):
    if rc != FPGM_OK:
        raise FpgmError(rc, load().fpgm_last_error().decode(errors="replace"))


def _u8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _i32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Engine:
    """One device context: dataset upload, CI tests and the PC-stable skeleton."""

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        _check(load().fpgm_engine_create(device, ctypes.byref(self._h)))
        self.n = 0
        self.S = 0

    def close(self):
        if self._h:
            load().fpgm_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, columns, relabel=True):
        """columns: uint8 [n_vars, n_samples] (C order = column-major samples).  Returns cardinalities."""
        columns = np.ascontiguousarray(columns, dtype=np.uint8)
        n, S = columns.shape
        card = np.zeros(n, dtype=np.uint8)
        _check(load().fpgm_dataset_upload(self._h, _u8(columns), n, S, 1 if relabel else 0, _u8(card)))
        self.n, self.S = n, S
        return card

    def upload_jobs(self, datasets, relabel=True):
        """Several independent datasets (uint8 [n_vars_j, n_samples_j] each) in one engine; the
        variables are numbered in dataset order.  Returns the per-dataset cardinalities."""
        datasets = [np.ascontiguousarray(c, dtype=np.uint8) for c in datasets]
        nv = np.array([c.shape[0] for c in datasets], dtype=np.int32)
        ns = np.array([c.shape[1] for c in datasets], dtype=np.int64)
        ptrs = (ctypes.c_void_p * len(datasets))(*[c.ctypes.data for c in datasets])
        card = np.zeros(int(nv.sum()), dtype=np.uint8)
        _check(load().fpgm_dataset_upload_jobs(self._h, len(datasets), _i32(nv),
                                               ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ptrs,
                                               1 if relabel else 0, _u8(card)))
        self.n, self.S = int(nv.sum()), int(ns.max())
        self.job_offsets = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
        return [card[self.job_offsets[j]:self.job_offsets[j + 1]] for j in range(len(datasets))]

    def mle_cpts(self, parents, alpha=1):
        """Maximum-likelihood tables with Laplace smoothing for a known DAG over the uploaded
        data.  parents: per variable an iterable of parent ids (order and repeats ignored).
        Returns a list of float64 arrays, variable v's over (v, sorted parents), v slowest."""
        off = [0]
        flat = []
        for p in parents:
            q = sorted(set(int(x) for x in p if int(x) >= 0))
            flat += q
            off.append(len(flat))
        off = np.array(off, dtype=np.int32)
        flat = np.array(flat if flat else [0], dtype=np.int32)
        toff = np.zeros(len(off), dtype=np.int64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        L = load()
        _check(L.fpgm_mle_cpts(self._h, _i32(off), _i32(flat), int(alpha), toff.ctypes.data_as(i64p), None))
        pot = np.zeros(int(toff[-1]), dtype=np.float64)
        _check(L.fpgm_mle_cpts(self._h, _i32(off), _i32(flat), int(alpha), toff.ctypes.data_as(i64p),
                               pot.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return [pot[toff[v]:toff[v + 1]] for v in range(len(off) - 1)]

    def download(self):
        out = np.empty((self.n, self.S), dtype=np.uint8)
        _check(load().fpgm_dataset_download(self._h, _u8(out)))
        return out

    def ci_test(self, x, y, z=(), alpha=0.05, want_hash=False):
        z = np.ascontiguousarray(list(z), dtype=np.int32)
        r = CIResult()
        _check(load().fpgm_ci_test(self._h, x, y, _i32(z) if len(z) else None, len(z), alpha, int(want_hash),
                                   ctypes.byref(r)))
        return r

    def ci_test_batch(self, tests, d, alpha=0.05, want_hash=False):
        tests = np.ascontiguousarray(tests, dtype=np.int32).reshape(-1, 2 + d)
        out = (CIResult * max(1, len(tests)))()
        _check(load().fpgm_ci_test_batch(self._h, _i32(tests), len(tests), d, alpha, int(want_hash), out))
        return [out[i] for i in range(len(tests))]

    def pc_skeleton(self, alpha=0.05, depth=1000, mode=FPGM_MODE_BATCHED):
        st = PCStats()
        _check(load().fpgm_pc_skeleton(self._h, alpha, depth, mode, ctypes.byref(st)))
        return st

    def result(self):
        """Returns dict(adj [n,n] uint8, removed [k,2] int32, sep_offsets, sep_vars, sepsets dict)."""
        r = self.result_arrays()
        off, var = r["sep_offsets"], r["sep_vars"]
        r["sepsets"] = {(int(a), int(b)): tuple(int(v) for v in var[off[k]:off[k + 1]])
                        for k, (a, b) in enumerate(r["removed"])}
        return r

    def result_arrays(self):
        """The skeleton as arrays only: adj [n,n] uint8, removed [k,2] int32, sep_offsets [k+1], sep_vars."""
        L = load()
        nn, nr, nv = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        _check(L.fpgm_pc_result_sizes(self._h, ctypes.byref(nn), ctypes.byref(nr), ctypes.byref(nv)))
        n = nn.value
        adj = np.zeros((n, n), dtype=np.uint8)
        removed = np.zeros((max(1, nr.value), 2), dtype=np.int32)
        off = np.zeros(nr.value + 1, dtype=np.int32)
        var = np.zeros(max(1, nv.value), dtype=np.int32)
        _check(L.fpgm_pc_result_fetch(self._h, _u8(adj), _i32(removed), _i32(off), _i32(var)))
        return {"adj": adj, "removed": removed[:nr.value], "sep_offsets": off, "sep_vars": var[:nv.value]}


def orient_cpdag(adj, removed, sep_offsets, sep_vars):
    """Host orientation; returns int32 [m, 3] edge records (a, b, directed) in the reference's order."""
    adj = np.ascontiguousarray(adj, dtype=np.uint8)
    n = adj.shape[0]
    removed = np.ascontiguousarray(removed, dtype=np.int32).reshape(-1, 2)
    sep_offsets = np.ascontiguousarray(sep_offsets, dtype=np.int32)
    sep_vars = np.ascontiguousarray(sep_vars, dtype=np.int32)
    if sep_vars.size == 0:
        sep_vars = np.zeros(1, dtype=np.int32)
    m = int(adj.sum()) // 2
    out = np.zeros((max(1, m + 64), 3), dtype=np.int32)
    cnt = ctypes.c_int32()
    _check(load().fpgm_orient_cpdag(n, _u8(adj), len(removed), _i32(removed), _i32(sep_offsets), _i32(sep_vars),
                                    _i32(out), ctypes.byref(cnt)))
    return out[:cnt.value]


def write_struct(path, names, edges, num_edges):
    n = len(names)
    arr = (ctypes.c_char_p * n)(*[s.encode() for s in names])
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 3)
    e = edges if len(edges) else np.zeros((1, 3), dtype=np.int32)
    _check(load().fpgm_write_struct(path.encode(), n, arr, _i32(e), len(edges), num_edges))


def generate(n_nodes, n_samples, seed, n_edges=0, avg_indegree=2.0, max_indegree=4, card=(2, 4),
             tail=(0.0, 2, 2), dirichlet=1.0):
    """Seeded random-DAG forward sample.  Returns (columns uint8 [n, S] raw ids, card, parents)."""
    spec = GenSpec(n_nodes, n_edges, avg_indegree, max_indegree, card[0], card[1], tail[0], tail[1], tail[2],
                   dirichlet, n_samples, seed)
    cols = np.empty((n_nodes, n_samples), dtype=np.uint8)
    c = np.empty(n_nodes, dtype=np.uint8)
    par = np.full((n_nodes, max(1, max_indegree)), -1, dtype=np.int32)
    _check(load().fpgm_generate_network(ctypes.byref(spec), _u8(cols), _u8(c), _i32(par)))
    return cols, c, par


def shd_bif(bif_path, n_nodes, edges):
    """Structural Hamming distance of learned edges ([m, 3] (a, b, directed), as orient_cpdag
    returns them) against the network of a BIF file, as BNSL_PCStable reports it."""
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 3)
    flat = edges if len(edges) else np.zeros((1, 3), dtype=np.int32)
    out = ctypes.c_int32()
    _check(load().fpgm_shd_bif(bif_path.encode(), int(n_nodes), _i32(flat), len(edges), ctypes.byref(out)))
    return out.value


def bnl_pcstable(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct, save_param):
    _check(load().fpgm_bnl_pcstable(verbose, n_threads, group_size, alpha, ref_net.encode(), train_set.encode(),
                                    int(bool(save_struct)), int(bool(save_param))))


def write_csv(path, columns, prefix="V"):
    columns = np.ascontiguousarray(columns, dtype=np.uint8)
    _check(load().fpgm_write_csv(path.encode(), _u8(columns), columns.shape[0], columns.shape[1], prefix.encode()))


def bnsl_pcstable(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct):
    _check(load().fpgm_bnsl_pcstable(verbose, n_threads, group_size, alpha, ref_net.encode(), train_set.encode(),
                                     int(bool(save_struct))))


from .configs import CONFIGS, c5_jobs, make_config, make_jobs, split_jobs  # noqa: E402
