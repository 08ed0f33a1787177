"""GPU: the BV and DS entry points of the C-ABI (the inner operations whose signatures the drop-in keeps), checked
against the reference's DS goldens and numpy."""
import ctypes
import json
import os

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen

pytestmark = pytest.mark.gpu
G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))
P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double


def setup_sigs(lib):
    sigs = {
        "DSCreate": [I, ctypes.POINTER(P)], "DSSetType": [P, ctypes.c_char_p], "DSAllocate": [P, I],
        "DSSetDimensions": [P, I, I, I], "DSSetCompact": [P, I], "DSSetExtraRow": [P, I], "DSSetState": [P, I],
        "DSGetArrayReal": [P, I, ctypes.POINTER(ctypes.POINTER(D))],
        "DSGetArray": [P, I, ctypes.POINTER(ctypes.POINTER(D))], "DSGetSlepcSC": [P, ctypes.POINTER(P)],
        "DSSolve": [P, P, P], "DSSort": [P, P, P, P, P, P], "DSUpdateExtraRow": [P], "DSVectors": [P, I, P, P],
        "DSDestroy": [ctypes.POINTER(P)],
        "BVCreate": [I, ctypes.POINTER(P)], "BVSetSizes": [P, I, I, I], "BVInsertVec": [P, I, P],
        "BVCopyVec": [P, I, P], "BVSetActiveColumns": [P, I, I], "BVDotVec": [P, P, P], "BVMultVec": [P, D, D, P, P],
        "BVMultInPlace": [P, P, I, I], "BVNormColumn": [P, I, I, P], "BVNorm": [P, I, P],
        "BVOrthonormalizeColumn": [P, I, I, P, P], "BVMatLanczos": [P, P, P, I, P, P, P],
        "BVMatArnoldi": [P, P, P, I, P, P, P], "BVDestroy": [ctypes.POINTER(P)],
        "MatCreateSeqDense": [I, I, I, P, ctypes.POINTER(P)],
    }
    for k, v in sigs.items():
        getattr(lib, k).argtypes = v
        getattr(lib, k).restype = I


DS_MAT_A, DS_MAT_T, DS_MAT_Q, DS_MAT_X = 0, 3, 5, 7


def test_ds_hep_golden_on_device(lib):
    setup_sigs(lib)
    g = G["ds_test3_1"]
    n, l, k = g["n"], g["l"], g["k"]
    ld = n + 2
    for extrarow in (False, True):
        ds = P()
        assert lib.DSCreate(0, ctypes.byref(ds)) == 0
        assert lib.DSSetType(ds, b"hep") == 0
        assert lib.DSAllocate(ds, ld) == 0
        assert lib.DSSetDimensions(ds, n, l, k) == 0
        assert lib.DSSetCompact(ds, 1) == 0
        assert lib.DSSetExtraRow(ds, int(extrarow)) == 0
        T = ctypes.POINTER(D)()
        assert lib.DSGetArrayReal(ds, DS_MAT_T, ctypes.byref(T)) == 0
        for i in range(n):
            T[i] = float(i + 1)
        for i in range(l, n - 1):
            T[i + ld] = 1.0
        if extrarow:
            T[n - 1 + ld] = 1.0
        assert lib.DSSetState(ds, 0) == 0
        sc = P()
        assert lib.DSGetSlepcSC(ds, ctypes.byref(sc)) == 0
        ctypes.cast(sc, ctypes.POINTER(P))[0] = ctypes.cast(lib.SlepcCompareLargestMagnitude, P).value
        eig = np.zeros(n)
        assert lib.DSSolve(ds, eig.ctypes.data_as(P), None) == 0
        assert lib.DSSort(ds, eig.ctypes.data_as(P), None, None, None, None) == 0
        assert [round(v, 5) for v in eig] == g["eigenvalues"]
        if extrarow:
            assert lib.DSUpdateExtraRow(ds) == 0
            Q = ctypes.POINTER(D)()
            assert lib.DSGetArray(ds, DS_MAT_Q, ctypes.byref(Q)) == 0
            assert lib.DSGetArrayReal(ds, DS_MAT_T, ctypes.byref(T)) == 0
            d = sum(T[i + ld] - Q[n - 1 + i * ld] for i in range(l, n))
            assert abs(d) < 10 * np.finfo(float).eps
        lib.DSDestroy(ctypes.byref(ds))


def test_ds_nhep_golden_on_device(lib):
    setup_sigs(lib)
    g = G["ds_test1_1"]
    n = g["n"]
    ld = n + 2
    ds = P()
    assert lib.DSCreate(0, ctypes.byref(ds)) == 0
    assert lib.DSSetType(ds, b"nhep") == 0
    assert lib.DSAllocate(ds, ld) == 0
    assert lib.DSSetDimensions(ds, n, 0, 0) == 0
    A = ctypes.POINTER(D)()
    assert lib.DSGetArray(ds, DS_MAT_A, ctypes.byref(A)) == 0
    for i in range(1, n):
        A[i + (i - 1) * ld] = -1.0
    for j in range(4):
        for i in range(n - j):
            A[i + (i + j) * ld] = 1.0
    assert lib.DSSetState(ds, 1) == 0
    sc = P()
    assert lib.DSGetSlepcSC(ds, ctypes.byref(sc)) == 0
    ctypes.cast(sc, ctypes.POINTER(P))[0] = ctypes.cast(lib.SlepcCompareLargestMagnitude, P).value
    wr, wi = np.zeros(n), np.zeros(n)
    assert lib.DSSolve(ds, wr.ctypes.data_as(P), wi.ctypes.data_as(P)) == 0
    assert lib.DSSort(ds, wr.ctypes.data_as(P), wi.ctypes.data_as(P), None, None, None) == 0
    got = [[round(a, 5), round(abs(b), 5)] for a, b in zip(wr, wi)]
    assert got == g["eigenvalues_abs_imag"]
    j = ctypes.c_int(2)
    rn = ctypes.c_double()
    assert lib.DSVectors(ds, DS_MAT_X, ctypes.byref(j), ctypes.byref(rn)) == 0
    assert round(rn.value, 3) == g["rnorm_3rd"]
    assert lib.DSVectors(ds, DS_MAT_X, None, None) == 0
    X = ctypes.POINTER(D)()
    assert lib.DSGetArray(ds, DS_MAT_X, ctypes.byref(X)) == 0
    nrm = np.hypot(np.linalg.norm([X[i] for i in range(n)]), np.linalg.norm([X[i + ld] for i in range(n)]))
    assert round(nrm, 3) == g["norm_1st"]
    lib.DSDestroy(ctypes.byref(ds))


def make_bv(lib, V):
    n, k = V.shape
    bv = P()
    assert lib.BVCreate(0, ctypes.byref(bv)) == 0
    assert lib.BVSetSizes(bv, n, n, k + 1) == 0
    keep = []
    for j in range(k):
        v = sg.Vec(np.ascontiguousarray(V[:, j]))
        keep.append(v)
        assert lib.BVInsertVec(bv, j, v.handle) == 0
    assert lib.BVSetActiveColumns(bv, 0, k) == 0
    return bv, keep


def test_bv_ops_against_numpy(lib):
    setup_sigs(lib)
    rng = np.random.default_rng(3)
    n, k = 3000, 12
    V = rng.standard_normal((n, k))
    bv, keep = make_bv(lib, V)
    x = rng.standard_normal(n)
    xv = sg.Vec(x)
    m = np.zeros(k)
    assert lib.BVDotVec(bv, xv.handle, m.ctypes.data_as(P)) == 0
    # dot-product error bound: proportional to sum |V_ij x_i|
    assert np.all(np.abs(m - V.T @ x) <= 1e-12 * (np.abs(V).T @ np.abs(x)))
    q = rng.standard_normal(k)
    y = rng.standard_normal(n)
    yv = sg.Vec(y.copy())
    assert lib.BVMultVec(bv, 0.5, 2.0, yv.handle, q.ctypes.data_as(P)) == 0
    assert np.all(np.abs(yv.array - (2.0 * y + 0.5 * V @ q)) <= 1e-12 * (2.0 * np.abs(y) + 0.5 * np.abs(V) @ np.abs(q)))
    nr = ctypes.c_double()
    assert lib.BVNormColumn(bv, 3, 1, ctypes.byref(nr)) == 0
    assert abs(nr.value - np.linalg.norm(V[:, 3])) < 1e-12 * np.linalg.norm(V[:, 3])
    assert lib.BVNorm(bv, 2, ctypes.byref(nr)) == 0  # Frobenius
    assert abs(nr.value - np.linalg.norm(V)) < 1e-12 * np.linalg.norm(V)
    # BVMultInPlace: V(:, 2:7) = V(:, 0:k) Q(:, 2:7)
    Qm = rng.standard_normal((k + 1, k + 1))
    Qf = np.asfortranarray(Qm)
    Qmat = P()
    assert lib.MatCreateSeqDense(0, k + 1, k + 1, Qf.ctypes.data_as(P), ctypes.byref(Qmat)) == 0
    assert lib.BVMultInPlace(bv, Qmat, 2, 7) == 0
    out = np.zeros(n)
    ov = sg.Vec(out)
    ref = V @ Qm[:k, 2:7]
    bound = np.abs(V) @ np.abs(Qm[:k, 2:7])
    for c in range(2, 7):
        assert lib.BVCopyVec(bv, c, ov.handle) == 0
        assert np.all(np.abs(ov.array - ref[:, c - 2]) <= 1e-12 * bound[:, c - 2])
    lib.BVDestroy(ctypes.byref(bv))


def test_bv_orthonormalize_and_lanczos(lib):
    setup_sigs(lib)
    rng = np.random.default_rng(5)
    n, m = 2000, 20
    bv = P()
    assert lib.BVCreate(0, ctypes.byref(bv)) == 0
    assert lib.BVSetSizes(bv, n, n, m + 1) == 0
    v0 = sg.Vec(rng.standard_normal(n))
    assert lib.BVInsertVec(bv, 0, v0.handle) == 0
    nrm, ld = ctypes.c_double(), ctypes.c_int()
    assert lib.BVOrthonormalizeColumn(bv, 0, 0, ctypes.byref(nrm), ctypes.byref(ld)) == 0
    assert abs(nrm.value - np.linalg.norm(v0.array)) < 1e-12 * nrm.value and ld.value == 0
    csr = matgen.laplacian_1d(n)
    A = sg.Mat(*csr)
    T = np.asfortranarray(np.zeros((m + 1, 2)))
    Tm = P()
    assert lib.MatCreateSeqDense(0, m + 1, 2, T.ctypes.data_as(P), ctypes.byref(Tm)) == 0
    mm, beta, bd = ctypes.c_int(m), ctypes.c_double(), ctypes.c_int()
    assert lib.BVMatLanczos(bv, A.handle, Tm, 0, ctypes.byref(mm), ctypes.byref(beta), ctypes.byref(bd)) == 0
    assert mm.value == m and bd.value == 0
    # A V = V T + beta v_m e_m^T with V orthonormal
    Vh = np.zeros((n, m + 1))
    col = sg.Vec(np.zeros(n))
    for j in range(m + 1):
        assert lib.BVCopyVec(bv, j, col.handle) == 0
        Vh[:, j] = col.array
    Ad = matgen.csr_to_dense(*csr)
    Tt = np.diag(T[:m, 0]) + np.diag(T[:m - 1, 1], 1) + np.diag(T[:m - 1, 1], -1)
    R = Ad @ Vh[:, :m] - Vh[:, :m] @ Tt
    R[:, m - 1] -= beta.value * Vh[:, m]
    assert np.abs(R).max() < 1e-12
    assert np.abs(Vh.T @ Vh - np.eye(m + 1)).max() < 1e-13
    lib.BVDestroy(ctypes.byref(bv))
