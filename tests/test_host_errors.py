"""The boundary's argument checks without a GPU: the PETSc error codes the reference's PetscCheck sites return
(epssetup.c:440-500 EPSSetOperators, epsopts.c EPSSet*, epsmon.c EPSMonitorSet), raised by the library before any
device work."""
import ctypes

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen

P = ctypes.c_void_p
PETSC_ERR_SUP, PETSC_ERR_ARG_WRONG, PETSC_ERR_ARG_OUTOFRANGE = 56, 62, 63
PETSC_ERR_ARG_WRONGSTATE, PETSC_ERR_ARG_INCOMP, PETSC_ERR_ARG_NULL = 73, 75, 85
PETSC_ERR_ARG_SIZ = 60


@pytest.fixture(scope="module")
def lib():
    sg.build()
    return sg.load()


def code(fn, *a):
    with pytest.raises(sg.SlepcError) as e:
        fn(*a)
    return e.value.code


def test_operator_checks(lib):
    eps = sg.EPS().create()
    A = sg.Mat(*matgen.laplacian_1d(10))
    B = sg.Mat(*matgen.diagonal(np.ones(12)))
    assert code(eps.setOperators, A, B) == PETSC_ERR_ARG_INCOMP        # "Dimensions of A and B do not match"
    rect = sg.Mat(np.array([0, 1, 2], np.int32), np.array([0, 2], np.int32), np.array([1.0, 2.0]), ncols=3)
    assert code(eps.setOperators, rect) == PETSC_ERR_ARG_WRONG        # "A does not have equal row and column sizes"
    empty = P()
    assert lib.MatCreate(0, ctypes.byref(empty)) == 0
    lib.EPSSetOperators.argtypes = [P, P, P]
    assert lib.EPSSetOperators(eps.handle, empty, None) == PETSC_ERR_ARG_WRONGSTATE  # MatCreate without MatLoad
    assert lib.EPSSetOperators(eps.handle, None, None) == PETSC_ERR_ARG_NULL
    assert lib.MatDestroy(ctypes.byref(empty)) == 0
    eps.setOperators(A, sg.Mat(*matgen.diagonal(np.ones(10))))        # a consistent pencil is accepted
    eps.destroy()


def test_setting_checks(lib):
    eps = sg.EPS().create()
    lib.EPSSetProblemType.argtypes = [P, ctypes.c_int]
    assert lib.EPSSetProblemType(eps.handle, 6) == PETSC_ERR_SUP       # EPS_GHIEP is not provided
    lib.EPSSetWhichEigenpairs.argtypes = [P, ctypes.c_int]
    assert lib.EPSSetWhichEigenpairs(eps.handle, 9) == PETSC_ERR_SUP   # EPS_TARGET_IMAGINARY
    assert lib.EPSSetWhichEigenpairs(eps.handle, 10) == PETSC_ERR_SUP  # EPS_ALL
    lib.EPSSetConvergenceTest.argtypes = [P, ctypes.c_int]
    assert lib.EPSSetConvergenceTest(eps.handle, 3) == PETSC_ERR_SUP   # EPS_CONV_USER
    assert lib.EPSSetConvergenceTest(eps.handle, 7) == PETSC_ERR_ARG_OUTOFRANGE
    lib.EPSKrylovSchurSetRestart.argtypes = [P, ctypes.c_double]
    assert lib.EPSKrylovSchurSetRestart(eps.handle, 0.95) == PETSC_ERR_ARG_OUTOFRANGE  # keep in [0.1, 0.9]
    lib.EPSSetExtraction.argtypes = [P, ctypes.c_int]
    assert lib.EPSSetExtraction(eps.handle, 5) == PETSC_ERR_SUP        # EPS_REFINED
    lib.EPSSetOptionsPrefix.argtypes = [P, ctypes.c_char_p]
    assert lib.EPSSetOptionsPrefix(eps.handle, b"-bad_") == PETSC_ERR_ARG_WRONG
    eps.setConvergenceTest("norm")
    assert eps.getConvergenceTest() == 2
    eps.destroy()


def test_queries_before_solve(lib):
    """Results before EPSSolve are an ordering error (EPSCheckSolved), as in the reference."""
    eps = sg.EPS().create()
    PETSC_ERR_ORDER = 58
    for f, args in (("EPSGetConverged", [P, P]), ("EPSGetConvergedReason", [P, P])):
        getattr(lib, f).argtypes = args
        out = ctypes.c_int()
        assert getattr(lib, f)(eps.handle, ctypes.byref(out)) == PETSC_ERR_ORDER
    lib.EPSComputeError.argtypes = [P, ctypes.c_int, ctypes.c_int, P]
    err = ctypes.c_double()
    assert lib.EPSComputeError(eps.handle, 0, 1, ctypes.byref(err)) == PETSC_ERR_ORDER
    eps.destroy()


def test_monitor_limit(lib):
    eps = sg.EPS().create()
    for _ in range(5):
        eps.monitorSet(lambda *a: None)
    with pytest.raises(sg.SlepcError) as e:
        eps.monitorSet(lambda *a: None)
    assert e.value.code == PETSC_ERR_ARG_OUTOFRANGE                    # "Too many EPS monitors set"
    eps.monitorCancel()
    eps.monitorSet(lambda *a: None)
    eps.destroy()


def test_balance_settings(lib):
    """EPSSetBalance/EPSGetBalance (epsopts.c:1062-1092) and -eps_balance*: stored as the reference stores them."""
    eps = sg.EPS().create()
    lib.EPSSetBalance.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    lib.EPSGetBalance.argtypes = [P, P, P, P]
    bal, its, cut = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()

    def get():
        assert lib.EPSGetBalance(eps.handle, ctypes.byref(bal), ctypes.byref(its), ctypes.byref(cut)) == 0
        return bal.value, its.value, cut.value

    assert get() == (0, 5, 1e-8)                                            # EPS_BALANCE_NONE, 5, 1e-8
    assert lib.EPSSetBalance(eps.handle, 1, 8, 1e-6) == 0 and get() == (1, 8, 1e-6)
    assert lib.EPSSetBalance(eps.handle, 2, -1, -1.0) == 0 and get() == (2, 5, 1e-8)   # PETSC_DETERMINE
    assert lib.EPSSetBalance(eps.handle, 2, -2, -2.0) == 0 and get() == (2, 5, 1e-8)   # PETSC_CURRENT
    assert lib.EPSSetBalance(eps.handle, 7, -2, -2.0) == PETSC_ERR_ARG_OUTOFRANGE
    assert lib.EPSSetBalance(eps.handle, 1, 0, -2.0) == PETSC_ERR_ARG_OUTOFRANGE        # its must be > 0
    eps.destroy()
    sg.initialize(["prog", "-eps_balance", "oneside", "-eps_balance_its", "3"])
    try:
        eps = sg.EPS().create()
        eps.setFromOptions()
        assert get() == (1, 3, 1e-8)
        eps.destroy()
    finally:
        sg.initialize(["prog"])


def test_gb300_setting_checks(lib):
    """The GB300 settings' argument checks: graph-capture mode, projected-solver method (the adaptive default among
    them), and EPSSetDeflationSpace (negative count, a null vector, vectors of different lengths); none needs the
    device."""
    eps = sg.EPS().create()
    lib.EPSGB300SetGraphCapture.argtypes = [P, ctypes.c_int]
    assert lib.EPSGB300SetGraphCapture(eps.handle, 2) == PETSC_ERR_ARG_OUTOFRANGE
    for mode in (-1, 0, 1):
        assert lib.EPSGB300SetGraphCapture(eps.handle, mode) == 0
    lib.EPSGB300SetProjectedSolver.argtypes = [P, ctypes.c_int]
    lib.EPSGB300GetProjectedSolver.argtypes = [P, P]
    m = ctypes.c_int(-1)
    assert lib.EPSGB300GetProjectedSolver(eps.handle, ctypes.byref(m)) == 0 and m.value == 2  # EPS_GB300_DS_AUTO
    assert lib.EPSGB300SetProjectedSolver(eps.handle, 3) == PETSC_ERR_ARG_OUTOFRANGE
    for meth in ("qr", "refined", "auto"):
        eps.setProjectedSolver(meth)
    # Gram-Schmidt methods: tensor 0, fma 1, integer 2, auto 3 (default)
    lib.EPSGB300SetGSMethod.argtypes = [P, ctypes.c_int]
    lib.EPSGB300GetGSMethod.argtypes = [P, P]
    assert lib.EPSGB300GetGSMethod(eps.handle, ctypes.byref(m)) == 0 and m.value == 3
    assert lib.EPSGB300SetGSMethod(eps.handle, 4) == PETSC_ERR_ARG_OUTOFRANGE
    for meth, val in (("tensor", 0), ("integer", 2), ("fma", 1), ("auto", 3)):
        eps.setGSMethod(meth)
        assert lib.EPSGB300GetGSMethod(eps.handle, ctypes.byref(m)) == 0 and m.value == val
    lib.EPSSetDeflationSpace.argtypes = [P, ctypes.c_int, P]
    assert lib.EPSSetDeflationSpace(eps.handle, -1, None) == PETSC_ERR_ARG_OUTOFRANGE
    assert lib.EPSSetDeflationSpace(eps.handle, 1, None) == PETSC_ERR_ARG_NULL
    v1, v2 = sg.Vec(np.ones(10)), sg.Vec(np.ones(12))
    arr = (P * 2)(v1.handle.value, v2.handle.value)
    assert lib.EPSSetDeflationSpace(eps.handle, 2, arr) == PETSC_ERR_ARG_SIZ
    eps.setDeflationSpace([np.ones(10), np.arange(10.0)])  # accepted; orthonormalised at set-up
    assert lib.EPSSetDeflationSpace(eps.handle, 0, None) == 0  # an empty space clears it
    eps.destroy()
