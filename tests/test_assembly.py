"""PETSc-style assembly on the host (MatCreate + MatSetSizes + MatSetValue(s) + MatAssemblyBegin/End, and the Vec
calls beside it) without a GPU: the matrices the reference's examples build with these calls come out as the same
CSR arrays as the generators the parity tests use, and the PETSc rules hold -- INSERT_VALUES replaces, ADD_VALUES
adds, negative indices are skipped, values and new nonzeros can be set between assemblies."""
import ctypes

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen

P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
INSERT_VALUES, ADD_VALUES = 1, 2
PETSC_DECIDE = -1


@pytest.fixture(scope="module")
def lib():
    sg.build()
    lib = sg.load()
    sigs = {
        "MatCreate": [I, ctypes.POINTER(P)], "MatSetSizes": [P, I, I, I, I], "MatSetFromOptions": [P],
        "MatSetUp": [P], "MatGetOwnershipRange": [P, ctypes.POINTER(I), ctypes.POINTER(I)],
        "MatSetValue": [P, I, I, D, I], "MatSetValues": [P, I, ctypes.POINTER(I), I, ctypes.POINTER(I),
                                                        ctypes.POINTER(D), I],
        "MatAssemblyBegin": [P, I], "MatAssemblyEnd": [P, I], "MatAssembled": [P, ctypes.POINTER(I)],
        "MatShift": [P, D], "MatScale": [P, D], "MatZeroEntries": [P], "MatDestroy": [ctypes.POINTER(P)],
        "MatGetRowIJ": [P, I, I, I, ctypes.POINTER(I), ctypes.POINTER(ctypes.POINTER(I)),
                        ctypes.POINTER(ctypes.POINTER(I)), ctypes.POINTER(I)],
        "MatSeqAIJGetArrayRead": [P, ctypes.POINTER(ctypes.POINTER(D))],
        "MatCreateSeqAIJWithArrays": [I, I, I, P, P, P, ctypes.POINTER(P)],
        "VecCreate": [I, ctypes.POINTER(P)], "VecSetSizes": [P, I, I], "VecSetFromOptions": [P],
        "VecSetValue": [P, I, D, I], "VecAssemblyBegin": [P], "VecAssemblyEnd": [P],
        "VecGetArray": [P, ctypes.POINTER(ctypes.POINTER(D))], "VecDestroy": [ctypes.POINTER(P)],
        "VecDuplicateVecs": [P, I, ctypes.POINTER(ctypes.POINTER(P))],
        "VecDestroyVecs": [I, ctypes.POINTER(ctypes.POINTER(P))], "VecPlaceArray": [P, ctypes.POINTER(D)],
        "VecResetArray": [P], "VecZeroEntries": [P], "VecGetSize": [P, ctypes.POINTER(I)],
    }
    for k, v in sigs.items():
        getattr(lib, k).argtypes = v
        getattr(lib, k).restype = I
    return lib


def new_mat(lib, m, n):
    A = P()
    assert lib.MatCreate(0, ctypes.byref(A)) == 0
    assert lib.MatSetSizes(A, PETSC_DECIDE, PETSC_DECIDE, m, n) == 0
    assert lib.MatSetFromOptions(A) == 0 and lib.MatSetUp(A) == 0
    return A


def csr_of(lib, A):
    n = I()
    ia, ja = ctypes.POINTER(I)(), ctypes.POINTER(I)()
    aa = ctypes.POINTER(D)()
    done = I()
    assert lib.MatGetRowIJ(A, 0, 0, 0, ctypes.byref(n), ctypes.byref(ia), ctypes.byref(ja), ctypes.byref(done)) == 0
    assert lib.MatSeqAIJGetArrayRead(A, ctypes.byref(aa)) == 0
    rp = np.ctypeslib.as_array(ia, (n.value + 1,)).copy()
    nnz = int(rp[-1])
    ci = np.ctypeslib.as_array(ja, (nnz,)).copy() if nnz else np.zeros(0, np.int32)
    va = np.ctypeslib.as_array(aa, (nnz,)).copy() if nnz else np.zeros(0)
    return rp, ci, va


def assemble(lib, A):
    assert lib.MatAssemblyBegin(A, 0) == 0 and lib.MatAssemblyEnd(A, 0) == 0


def test_ex2_laplacian_as_the_reference_builds_it(lib):
    """ex2.c's loop (src/eps/tutorials/ex2.c:54-66): the 2-D Laplacian N x M, rows in the ownership range."""
    N = M = 9
    A = new_mat(lib, N * M, N * M)
    rs, re = I(), I()
    assert lib.MatGetOwnershipRange(A, ctypes.byref(rs), ctypes.byref(re)) == 0 and (rs.value, re.value) == (0, 81)
    for II in range(rs.value, re.value):
        i, j = II // N, II - (II // N) * N
        if i > 0:
            lib.MatSetValue(A, II, II - N, -1.0, INSERT_VALUES)
        if i < M - 1:
            lib.MatSetValue(A, II, II + N, -1.0, INSERT_VALUES)
        if j > 0:
            lib.MatSetValue(A, II, II - 1, -1.0, INSERT_VALUES)
        if j < N - 1:
            lib.MatSetValue(A, II, II + 1, -1.0, INSERT_VALUES)
        lib.MatSetValue(A, II, II, 4.0, INSERT_VALUES)
    flag = I(-1)
    assert lib.MatAssembled(A, ctypes.byref(flag)) == 0 and flag.value == 0
    assemble(lib, A)
    assert lib.MatAssembled(A, ctypes.byref(flag)) == 0 and flag.value == 1
    rp, ci, va = csr_of(lib, A)
    ref = matgen.laplacian_2d(N, M)
    assert np.array_equal(rp, ref[0]) and np.array_equal(ci, ref[1]) and np.array_equal(va, ref[2])
    assert lib.MatDestroy(ctypes.byref(A)) == 0


def test_insert_add_negative_and_reassembly(lib):
    A = new_mat(lib, 3, 4)
    lib.MatSetValue(A, 0, 2, 5.0, INSERT_VALUES)
    lib.MatSetValue(A, 0, 2, 7.0, INSERT_VALUES)       # the last insert wins
    lib.MatSetValue(A, 2, 1, 1.5, ADD_VALUES)
    lib.MatSetValue(A, 2, 1, 2.0, ADD_VALUES)          # adds
    rows, cols = (I * 2)(1, -1), (I * 2)(3, 0)         # a negative row is skipped
    vals = (D * 4)(1.0, 2.0, 3.0, 4.0)
    assert lib.MatSetValues(A, 2, rows, 2, cols, vals, INSERT_VALUES) == 0
    assert lib.MatSetValue(A, 3, 0, 1.0, INSERT_VALUES) == 63   # row out of range
    assemble(lib, A)
    rp, ci, va = csr_of(lib, A)
    assert rp.tolist() == [0, 1, 3, 4] and ci.tolist() == [2, 0, 3, 1] and va.tolist() == [7.0, 2.0, 1.0, 3.5]
    lib.MatSetValue(A, 1, 3, 10.0, ADD_VALUES)         # after assembly: change a value, add a nonzero
    lib.MatSetValue(A, 0, 0, -1.0, INSERT_VALUES)
    assemble(lib, A)
    rp, ci, va = csr_of(lib, A)
    assert rp.tolist() == [0, 2, 4, 5] and ci.tolist() == [0, 2, 0, 3, 1] and va.tolist() == [-1.0, 7.0, 2.0, 11.0, 3.5]
    assert lib.MatDestroy(ctypes.byref(A)) == 0


def test_shift_scale_zero_and_caller_arrays(lib):
    rp = np.array([0, 1, 2, 3], np.int32)
    ci = np.array([1, 2, 0], np.int32)
    va = np.array([1.0, 2.0, 3.0])
    A = P()
    assert lib.MatCreateSeqAIJWithArrays(0, 3, 3, rp.ctypes.data, ci.ctypes.data, va.ctypes.data, ctypes.byref(A)) == 0
    assert lib.MatShift(A, 0.5) == 0                   # adds the missing diagonal
    r, c, v = csr_of(lib, A)
    assert r.tolist() == [0, 2, 4, 6] and c.tolist() == [0, 1, 1, 2, 0, 2]
    assert v.tolist() == [0.5, 1.0, 0.5, 2.0, 3.0, 0.5]
    assert lib.MatScale(A, 2.0) == 0
    assert csr_of(lib, A)[2].tolist() == [1.0, 2.0, 1.0, 4.0, 6.0, 1.0]
    assert va.tolist() == [1.0, 2.0, 3.0]              # the caller's arrays are left as they were
    assert lib.MatZeroEntries(A) == 0 and not np.any(csr_of(lib, A)[2])
    assert lib.MatDestroy(ctypes.byref(A)) == 0


def test_unassembled_matrix_is_rejected(lib):
    A = new_mat(lib, 4, 4)
    lib.MatSetValue(A, 0, 0, 1.0, INSERT_VALUES)
    eps = sg.EPS().create()
    lib.EPSSetOperators.argtypes = [P, P, P]
    assert lib.EPSSetOperators(eps.handle, A, None) == 73   # "Not for unassembled matrix"
    assemble(lib, A)
    assert lib.EPSSetOperators(eps.handle, A, None) == 0
    eps.destroy()
    assert lib.MatDestroy(ctypes.byref(A)) == 0


def test_vec_calls(lib):
    x = P()
    assert lib.VecCreate(0, ctypes.byref(x)) == 0
    assert lib.VecSetSizes(x, PETSC_DECIDE, 5) == 0 and lib.VecSetFromOptions(x) == 0
    lib.VecSetValue(x, 1, 2.0, INSERT_VALUES)
    lib.VecSetValue(x, 1, 3.0, ADD_VALUES)
    lib.VecSetValue(x, -1, 9.0, INSERT_VALUES)         # skipped
    assert lib.VecAssemblyBegin(x) == 0 and lib.VecAssemblyEnd(x) == 0
    a = ctypes.POINTER(D)()
    assert lib.VecGetArray(x, ctypes.byref(a)) == 0
    assert [a[i] for i in range(5)] == [0.0, 5.0, 0.0, 0.0, 0.0]
    vs = ctypes.POINTER(P)()
    assert lib.VecDuplicateVecs(x, 3, ctypes.byref(vs)) == 0
    n = I()
    assert lib.VecGetSize(P(vs[2]), ctypes.byref(n)) == 0 and n.value == 5
    assert lib.VecDestroyVecs(3, ctypes.byref(vs)) == 0 and not vs
    buf = (D * 5)(*range(5))
    assert lib.VecPlaceArray(x, buf) == 0
    assert lib.VecGetArray(x, ctypes.byref(a)) == 0 and a[3] == 3.0
    assert lib.VecPlaceArray(x, buf) == 73              # placed twice
    assert lib.VecResetArray(x) == 0 and lib.VecGetArray(x, ctypes.byref(a)) == 0 and a[1] == 5.0
    assert lib.VecZeroEntries(x) == 0 and lib.VecGetArray(x, ctypes.byref(a)) == 0 and a[1] == 0.0
    assert lib.VecDestroy(ctypes.byref(x)) == 0
