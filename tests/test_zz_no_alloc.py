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
