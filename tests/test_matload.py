"""PETSc binary files: MatLoad/MatView/VecLoad/VecView against an independent numpy reader/writer of the format,
error codes on damaged files, and the reference's real matrix rdb200 (share/slepc/datafiles/matrices/rdb200.petsc,
converted to tests/golden/rdb200.npz) solved by the oracle to the digits of src/eps/tutorials/output/ex4_1.out."""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle
import slepc_gb300 as sg
from slepc_gb300 import matgen

HERE = os.path.dirname(os.path.abspath(__file__))
G = json.load(open(os.path.join(HERE, "golden", "reference_outputs.json")))

PETSC_ERR_FILE_OPEN, PETSC_ERR_FILE_READ, PETSC_ERR_FILE_UNEXPECTED = 65, 66, 79
PETSC_ERR_ARG_WRONGSTATE = 73


def rdb200():
    d = np.load(os.path.join(HERE, "golden", "rdb200.npz"))
    return d["rowptr"], d["colidx"], d["vals"]


def write_petsc(path, rowptr, colidx, vals, m=None, n=None):
    """PETSc's binary matrix layout written with numpy big-endian dtypes (independent of the library)."""
    m = len(rowptr) - 1 if m is None else m
    n = m if n is None else n
    with open(path, "wb") as f:
        f.write(np.array([1211216, m, n, len(colidx)], dtype=">i4").tobytes())
        f.write(np.diff(rowptr).astype(">i4").tobytes())
        f.write(np.asarray(colidx).astype(">i4").tobytes())
        f.write(np.asarray(vals).astype(">f8").tobytes())


@pytest.fixture(scope="module")
def lib():
    sg.build()
    return sg.load()


def test_matload_reads_the_format(lib, tmp_path):
    rp, ci, va = rdb200()
    p = tmp_path / "a.petsc"
    write_petsc(p, rp, ci, va)
    A = sg.Mat.load(str(p))
    assert A.m == A.n == 200
    assert np.array_equal(A.rowptr, rp) and np.array_equal(A.colidx, ci) and np.array_equal(A.vals, va)


def test_matview_writes_the_same_bytes(lib, tmp_path):
    rp, ci, va = rdb200()
    ours, ref = tmp_path / "ours.petsc", tmp_path / "ref.petsc"
    sg.Mat(rp, ci, va).save(str(ours))
    write_petsc(ref, rp, ci, va)
    assert ours.read_bytes() == ref.read_bytes()
    B = sg.Mat.load(str(ours))
    assert np.array_equal(B.vals, va)


def test_rectangular_and_empty_rows(lib, tmp_path):
    rp = np.array([0, 2, 2, 3], dtype=np.int32)  # row 1 empty
    ci = np.array([0, 4, 1], dtype=np.int32)
    va = np.array([1.5, -2.0, 3.25])
    p = tmp_path / "r.petsc"
    write_petsc(p, rp, ci, va, m=3, n=5)
    A = sg.Mat.load(str(p))
    assert (A.m, A.n) == (3, 5)
    assert np.array_equal(A.rowptr, rp) and np.array_equal(A.colidx, ci) and np.array_equal(A.vals, va)


def test_vec_round_trip(lib, tmp_path):
    x = matgen.start_vector(37, 5)
    p = str(tmp_path / "v.petsc").encode()
    viewer, v, w = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    assert lib.VecCreateSeqWithArray(0, 1, 37, x.ctypes.data_as(ctypes.c_void_p), ctypes.byref(v)) == 0
    assert lib.PetscViewerBinaryOpen(0, p, 1, ctypes.byref(viewer)) == 0
    assert lib.VecView(v, viewer) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(viewer)) == 0
    raw = open(p, "rb").read()
    assert np.array_equal(np.frombuffer(raw[:8], ">i4"), [1211214, 37])
    assert np.array_equal(np.frombuffer(raw[8:], ">f8"), x)
    assert lib.VecCreateSeq(0, 37, ctypes.byref(w)) == 0
    assert lib.PetscViewerBinaryOpen(0, p, 0, ctypes.byref(viewer)) == 0
    assert lib.VecLoad(w, viewer) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(viewer)) == 0
    arr = ctypes.POINTER(ctypes.c_double)()
    assert lib.VecGetArray(w, ctypes.byref(arr)) == 0
    assert np.array_equal(np.ctypeslib.as_array(arr, (37,)), x)
    lib.VecDestroy(ctypes.byref(v))
    lib.VecDestroy(ctypes.byref(w))


def _load_rc(lib, path):
    viewer, h = ctypes.c_void_p(), ctypes.c_void_p()
    rc = lib.PetscViewerBinaryOpen(0, str(path).encode(), 0, ctypes.byref(viewer))
    if rc:
        return rc
    lib.MatCreate(0, ctypes.byref(h))
    rc = lib.MatLoad(h, viewer)
    lib.PetscViewerDestroy(ctypes.byref(viewer))
    lib.MatDestroy(ctypes.byref(h))
    return rc


def test_damaged_files_are_errors(lib, tmp_path):
    rp, ci, va = rdb200()
    good = tmp_path / "g.petsc"
    write_petsc(good, rp, ci, va)
    raw = good.read_bytes()
    assert _load_rc(lib, tmp_path / "missing.petsc") == PETSC_ERR_FILE_OPEN
    cut = tmp_path / "cut.petsc"
    cut.write_bytes(raw[:-8])
    assert _load_rc(lib, cut) == PETSC_ERR_FILE_READ
    bad = tmp_path / "bad.petsc"
    bad.write_bytes(np.array([1211214], ">i4").tobytes() + raw[4:])  # a vector's class id
    assert _load_rc(lib, bad) == PETSC_ERR_FILE_UNEXPECTED
    col = bytearray(raw)
    col[16 + 4 * 200: 16 + 4 * 200 + 4] = np.array([200], ">i4").tobytes()  # column index out of range
    badc = tmp_path / "badc.petsc"
    badc.write_bytes(bytes(col))
    assert _load_rc(lib, badc) == PETSC_ERR_FILE_UNEXPECTED


def test_empty_mat_is_rejected_by_the_solver(lib):
    h, eps = ctypes.c_void_p(), ctypes.c_void_p()
    assert lib.MatCreate(0, ctypes.byref(h)) == 0
    assert lib.EPSCreate(0, ctypes.byref(eps)) == 0
    assert lib.EPSSetOperators(eps, h, None) == PETSC_ERR_ARG_WRONGSTATE
    lib.EPSDestroy(ctypes.byref(eps))
    lib.MatDestroy(ctypes.byref(h))


def test_oracle_reproduces_ex4_on_rdb200():
    """ex4 -file rdb200.petsc -eps_nev 4: EPS_NHEP (no problem type set), largest magnitude, tol 1e-8, default ncv."""
    g = G["ex4_1"]
    oracle.build()
    rp, ci, va = rdb200()
    r = oracle.solve(rp, ci, va, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"],
                     v0=matgen.start_vector(200, 1))
    assert r.err == 0 and r.reason == 1
    assert np.all(np.asarray(r.eigi[:4]) == 0.0)
    assert [round(v, 5) for v in r.eigr[:4]] == g["eigenvalues"]
