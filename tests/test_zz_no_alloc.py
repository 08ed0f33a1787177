"""BVGB300DotVecNoAlloc -- the dot kernel with its scratch in a static device array, for callers that cannot
allocate device memory while they run -- checked through the C-ABI against BVDotVec, twice in a row (the second
call must not see the first call's scratch contents); after those warm-up calls, more calls leave the device's free
memory unchanged; bad sizes and alignment are refused with an error.  This file is named to run last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H2D, D2H = 1, 2


def _cudart():
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    rt.cudaDeviceSynchronize.argtypes = []
    rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    return rt


def _free_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def _bvdotvec(lib, V, x):
    n, k = V.shape
    P, I = ctypes.c_void_p, ctypes.c_int
    lib.BVCreate.argtypes = [I, ctypes.POINTER(P)]
    lib.BVSetSizes.argtypes = [P, I, I, I]
    lib.BVInsertVec.argtypes = [P, I, P]
    lib.BVDotVec.argtypes = [P, P, P]
    lib.BVSetActiveColumns.argtypes = [P, I, I]
    lib.BVDestroy.argtypes = [ctypes.POINTER(P)]
    import slepc_gb300 as sg
    bv = P()
    assert lib.BVCreate(0, ctypes.byref(bv)) == 0
    assert lib.BVSetSizes(bv, n, n, k) == 0
    cols = [sg.Vec(np.ascontiguousarray(V[:, j])) for j in range(k)]
    for j, c in enumerate(cols):
        assert lib.BVInsertVec(bv, j, c.handle) == 0
    assert lib.BVSetActiveColumns(bv, 0, k) == 0
    xv = sg.Vec(x)
    m = np.zeros(k)
    assert lib.BVDotVec(bv, xv.handle, m.ctypes.data_as(P)) == 0
    lib.BVDestroy(ctypes.byref(bv))
    return m


def test_no_alloc_dot_matches_bvdotvec(lib):
    rt = _cudart()
    f = lib.BVGB300DotVecNoAlloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(11)
    n, k = 20000, 37
    V = np.asfortranarray(rng.standard_normal((n, k)))
    dV, dx, dy = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dV), V.nbytes) == 0
    assert rt.cudaMalloc(ctypes.byref(dx), n * 8) == 0
    assert rt.cudaMalloc(ctypes.byref(dy), k * 8) == 0
    try:
        assert rt.cudaMemcpy(dV, V.ctypes.data, V.nbytes, H2D) == 0
        for call in range(2):
            x = rng.standard_normal(n) * (1.0 + call)
            assert rt.cudaMemcpy(dx, x.ctypes.data, n * 8, H2D) == 0
            assert f(dV, n, n, k, dx, dy, None) == 0
            assert rt.cudaDeviceSynchronize() == 0
            y = np.zeros(k)
            assert rt.cudaMemcpy(y.ctypes.data, dy, k * 8, D2H) == 0
            ref = _bvdotvec(lib, V, x)
            scale = np.abs(V).T @ np.abs(x)
            assert np.all(np.abs(y - ref) <= 1e-13 * scale), (call, np.max(np.abs(y - ref) / scale))
            assert np.all(np.abs(y - V.T @ x) <= 1e-12 * scale)
        # after the warm-up calls above, further calls allocate no device memory
        before = _free_bytes(rt)
        for _ in range(4):
            assert f(dV, n, n, k, dx, dy, None) == 0
            assert rt.cudaDeviceSynchronize() == 0
        assert _free_bytes(rt) == before
        # sizes beyond the fixed scratch, an odd leading dimension and a V that is not 16-byte aligned are refused
        # with an error before any launch
        assert f(dV, n, n, 257, dx, dy, None) != 0
        assert f(dV, n + 1, n, k, dx, dy, None) != 0
        assert f(ctypes.c_void_p(dV.value + 8), n, n, k, dx, dy, None) != 0
        assert rt.cudaDeviceSynchronize() == 0
    finally:
        rt.cudaFree(dV)
        rt.cudaFree(dx)
        rt.cudaFree(dy)
