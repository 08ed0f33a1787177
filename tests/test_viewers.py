"""ASCII viewers and the EPS text reports without a GPU: the format stack, PetscViewerASCIIPrintf, the stdout viewer,
EPSConvergedReasonView of an EPS that has not run (epsview.c:243-262 prints CONVERGED_ITERATING with 0 iterations),
EPSErrorView before EPSSolve (PETSC_ERR_ORDER) and binary calls on an ASCII viewer (PETSC_ERR_SUP).  The reports
of solved problems are checked against the reference's printed text in test_gpu_eps.py."""
import ctypes

import pytest

import slepc_gb300 as sg

P = ctypes.c_void_p
PETSC_ERR_SUP, PETSC_ERR_ORDER = 56, 58
PETSC_VIEWER_DEFAULT, PETSC_VIEWER_ASCII_INFO_DETAIL = 0, 5


@pytest.fixture(scope="module")
def lib():
    sg.build()
    lib = sg.load()
    lib.PETSC_VIEWER_STDOUT_.restype = P
    lib.PETSC_VIEWER_STDOUT_.argtypes = [ctypes.c_int]
    lib.PetscViewerGetFormat.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    lib.PetscViewerASCIIGetStdout.argtypes = [ctypes.c_int, ctypes.POINTER(P)]
    lib.MatLoad.argtypes = [P, P]
    return lib


def open_ascii(lib, path):
    v = P()
    assert lib.PetscViewerASCIIOpen(0, str(path).encode(), ctypes.byref(v)) == 0
    return v


def test_format_stack_and_printf(lib, tmp_path):
    path = tmp_path / "out.txt"
    v = open_ascii(lib, path)
    fmt = ctypes.c_int(-1)
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT
    assert lib.PetscViewerPushFormat(v, PETSC_VIEWER_ASCII_INFO_DETAIL) == 0
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_ASCII_INFO_DETAIL
    assert lib.PetscViewerPopFormat(v) == 0
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT
    assert lib.PetscViewerASCIIPrintf(v, b"n=%d x=%.3f\n", ctypes.c_int(30), ctypes.c_double(2.5)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0 and not v.value
    assert path.read_text() == "n=30 x=2.500\n"


def test_stdout_viewer_is_shared_and_not_closed(lib):
    a = lib.PETSC_VIEWER_STDOUT_(0)
    b = P()
    assert lib.PetscViewerASCIIGetStdout(1, ctypes.byref(b)) == 0
    assert a and a == b.value
    assert lib.PetscViewerDestroy(ctypes.byref(b)) == 0 and not b.value
    fmt = ctypes.c_int(-1)
    assert lib.PetscViewerGetFormat(P(a), ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT


def test_reports_before_solve(lib, tmp_path):
    eps = sg.EPS().create()
    assert eps.convergedReasonView() == (" Linear eigensolve did not converge due to CONVERGED_ITERATING; "
                                         "iterations 0\n")
    with pytest.raises(sg.SlepcError) as e:
        eps.errorView()
    assert e.value.code == PETSC_ERR_ORDER
    with pytest.raises(sg.SlepcError) as e:
        eps.valuesView()
    assert e.value.code == PETSC_ERR_ORDER
    eps.destroy()


def test_binary_calls_reject_ascii_viewers(lib, tmp_path):
    v = open_ascii(lib, tmp_path / "m.txt")
    A = P()
    assert lib.MatCreate(0, ctypes.byref(A)) == 0
    assert lib.MatLoad(A, v) == PETSC_ERR_SUP
    assert lib.MatDestroy(ctypes.byref(A)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0
