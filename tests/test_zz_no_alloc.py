"""The allocation-free CI test entry point (fpgm_ci_test_noalloc) against fpgm_ci_test.

Some callers cannot allocate device memory -- their device memory is owned by another
allocator, or cudaMalloc is not allowed where they run -- so the library offers one CI
test that works only on the caller's device buffers and a fixed scratch array inside the
library.  This checks, through the C ABI, that it returns what the ordinary (allocating)
entry point returns, on two calls in a row (the scratch array is reused), and that a
table beyond its fixed limit is refused.  Kept in a file of its own that pytest collects
last.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
import fastpgm_gb300 as F

pytestmark = pytest.mark.gpu

# tolerances of tests/test_gpu_ci.py: FP32-compensated G^2 vs FP64, and p outside the band
G2_RTOL, G2_ATOL = 2e-5, 2e-3
P_ATOL = 1e-3


def _device_copy(torch, arr, pitch):
    n, S = arr.shape
    buf = torch.zeros((n, pitch), dtype=torch.uint8, device="cuda:0")
    buf[:, :S] = torch.from_numpy(np.ascontiguousarray(arr))
    return buf


def test_noalloc_matches_ci_test_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = F.load()
    raw, _, _ = F.generate(n_nodes=16, n_samples=5003, seed=21, n_edges=22, max_indegree=3, card=(2, 5))
    with F.Engine(0) as eng:
        eng.upload(raw)                 # first-appearance ids on the device
        cols = eng.download()
        n, S = cols.shape
        pitch = (S + 63) // 64 * 64
        dcols = _device_copy(torch, cols, pitch)
        dres = torch.zeros(ctypes.sizeof(F.CIResult), dtype=torch.uint8, device="cuda:0")
        rng = np.random.default_rng(4)
        tests = [tuple(int(v) for v in rng.choice(n, size=2 + d, replace=False)) for d in (0, 1, 2, 3) for _ in range(6)]
        for call in range(2):
            for t in tests:
                x, y, z = t[0], t[1], list(t[2:])
                zarr = np.array(z if z else [0], dtype=np.int32)
                rc = lib.fpgm_ci_test_noalloc(dcols.data_ptr(), pitch, n, S, x, y,
                                              zarr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(z), 0.05, 1,
                                              dres.data_ptr(), None)
                assert rc == 0, lib.fpgm_last_error()
                torch.cuda.synchronize()
                got = F.CIResult.from_buffer_copy(dres.cpu().numpy().tobytes())
                exp = eng.ci_test(x, y, z, want_hash=True)
                assert got.table_hash == exp.table_hash and got.cell_hash == exp.cell_hash, (call, t)
                assert got.df == exp.df and got.independent == exp.independent, (call, t)
                assert abs(got.g2 - exp.g2) <= max(G2_ATOL, G2_RTOL * abs(exp.g2)), (call, t)
                tol = 1e-10 if exp.rechecked else P_ATOL
                assert abs(got.p_value - exp.p_value) <= tol, (call, t)
                _check_oracle(got, cols, t)


def _check_oracle(got, cols, t):
    """The CPU oracle's counts (table hash), df, decision and FP64 G^2 / p for the same test."""
    card = (cols.max(axis=1).astype(np.int32) + 1).astype(np.uint8)  # dense ids: card = max + 1
    o = O.ci_tests(cols, card, np.array([t], dtype=np.int32), len(t) - 2, threads=1)[0]
    assert got.table_hash == o.table_hash and got.cell_hash == o.cell_hash, t
    assert got.df == o.df and got.independent == o.independent, t
    assert abs(got.g2 - o.g2) <= max(G2_ATOL, G2_RTOL * abs(o.g2)), t
    assert abs(got.p_value - o.p_value) <= (1e-10 if got.rechecked else P_ATOL), t


def test_noalloc_large_table_on_a_stream():
    """A joint table of 140,000+ cells (beyond the shared-memory table, so the kernel counts
    into the library's fixed scratch array with global atomics), issued on a caller's
    non-default stream: the same result as fpgm_ci_test and the oracle, on two calls in a row."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = F.load()
    raw, _, _ = F.generate(n_nodes=8, n_samples=30011, seed=31, n_edges=9, max_indegree=2, card=(18, 20))
    with F.Engine(0) as eng:
        eng.upload(raw)
        cols = eng.download()
        n, S = cols.shape
        pitch = (S + 63) // 64 * 64
        dcols = _device_copy(torch, cols, pitch)
        dres = torch.zeros(ctypes.sizeof(F.CIResult), dtype=torch.uint8, device="cuda:0")
        stream = torch.cuda.Stream()
        tests = [(0, 1, 2, 3), (4, 5, 6, 7), (2, 6, 0, 5)]
        for call in range(2):
            for t in tests:
                card = cols.max(axis=1).astype(np.int64) + 1
                assert np.prod(card[list(t)]) > 24576  # beyond the shared-memory table
                z = np.array(t[2:], dtype=np.int32)
                rc = lib.fpgm_ci_test_noalloc(dcols.data_ptr(), pitch, n, S, t[0], t[1],
                                              z.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 2, 0.05, 1,
                                              dres.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
                assert rc == 0, lib.fpgm_last_error()
                stream.synchronize()
                got = F.CIResult.from_buffer_copy(dres.cpu().numpy().tobytes())
                exp = eng.ci_test(t[0], t[1], list(t[2:]), want_hash=True)
                assert got.table_hash == exp.table_hash and got.df == exp.df, (call, t)
                assert got.independent == exp.independent, (call, t)
                assert abs(got.g2 - exp.g2) <= max(G2_ATOL, G2_RTOL * abs(exp.g2)), (call, t)
                _check_oracle(got, cols, t)


def test_noalloc_rejects_a_misaligned_result():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = F.load()
    cols = np.zeros((2, 64), dtype=np.uint8)
    dcols = _device_copy(torch, cols, 64)
    dres = torch.zeros(ctypes.sizeof(F.CIResult) + 16, dtype=torch.uint8, device="cuda:0")
    rc = lib.fpgm_ci_test_noalloc(dcols.data_ptr(), 64, 2, 64, 0, 1, None, 0, 0.05, 0, dres.data_ptr() + 4, None)
    assert rc == F.FPGM_ERR_INVALID
    assert b"aligned" in lib.fpgm_last_error()


def test_noalloc_rejects_tables_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = F.load()
    rng = np.random.default_rng(9)
    S = 4096
    cols = rng.integers(0, 40, size=(6, S)).astype(np.uint8)   # 40^6 cells, far beyond 2^20
    dcols = _device_copy(torch, cols, S)
    dres = torch.zeros(ctypes.sizeof(F.CIResult), dtype=torch.uint8, device="cuda:0")
    z = np.array([2, 3, 4, 5], dtype=np.int32)
    rc = lib.fpgm_ci_test_noalloc(dcols.data_ptr(), S, 6, S, 0, 1, z.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 4,
                                  0.05, 0, dres.data_ptr(), None)
    assert rc == F.FPGM_ERR_UNSUPPORTED if hasattr(F, "FPGM_ERR_UNSUPPORTED") else rc == -6
    assert b"scratch" in lib.fpgm_last_error()
