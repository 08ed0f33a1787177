"""slepc_gb300 -- GB300-native Krylov-Schur eigensolver behind SLEPc's API.

The product is the C-ABI library ``_build/libslepc_gb300.so`` (hand-written sm_103a CUDA kernels plus the C++ host
driver; headers in ``include/``).  This module is the Python host mirror of slepc4py's EPS/Mat/Vec interface for
that path (``src/binding/slepc4py/SLEPc/EPS.pyx``: ``setOperators`` :1087, ``solve`` :1290, ``getEigenpair``
:1426), implemented over ctypes.  There is no CPU fallback: loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libslepc_gb300.so")

_lib = None


class SlepcError(RuntimeError):
    def __init__(self, code, where, msg):
        super().__init__(f"{where} failed with PETSc error {code}: {msg}")
        self.code = code


def build(force=False, verbose=False):
    from . import buildlib as _b
    return _b.build(force=force, verbose=verbose)


def load():
    """Load libslepc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"slepc_gb300 CUDA library not built ({LIB_PATH}); run slepc_gb300.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    PP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "PetscGB300LastError": ([], ctypes.c_char_p),
        "MatCreateSeqAIJWithArrays": ([I, I, I, P, P, P, PP], I),
        "MatCreateSeqDense": ([I, I, I, P, PP], I),
        "MatDestroy": ([PP], I),
        "MatMult": ([P, P, P], I),
        "VecCreateSeqWithArray": ([I, I, I, P, PP], I),
        "VecDestroy": ([PP], I),
        "EPSCreate": ([I, PP], I),
        "EPSDestroy": ([PP], I),
        "EPSSetOperators": ([P, P, P], I),
        "EPSSetProblemType": ([P, I], I),
        "EPSSetType": ([P, ctypes.c_char_p], I),
        "EPSSetDimensions": ([P, I, I, I], I),
        "EPSGetDimensions": ([P, P, P, P], I),
        "EPSSetTolerances": ([P, D, I], I),
        "EPSGetTolerances": ([P, P, P], I),
        "EPSSetWhichEigenpairs": ([P, I], I),
        "EPSSetInitialSpace": ([P, I, PP], I),
        "EPSKrylovSchurSetRestart": ([P, D], I),
        "EPSKrylovSchurSetLocking": ([P, I], I),
        "EPSSetUp": ([P], I),
        "EPSSolve": ([P], I),
        "EPSGetConverged": ([P, P], I),
        "EPSGetConvergedReason": ([P, P], I),
        "EPSGetIterationNumber": ([P, P], I),
        "EPSGetEigenpair": ([P, I, P, P, P, P], I),
        "EPSGetEigenvalue": ([P, I, P, P], I),
        "EPSGetErrorEstimate": ([P, I, P], I),
        "EPSComputeError": ([P, I, I, P], I),
        "EPSGB300SetArithmetic": ([P, I], I),
        "EPSGB300SetProjectedSolver": ([P, I], I),
        "EPSGB300SolveBatch": ([I, ctypes.POINTER(P)], I),
        "EPSGB300BatchTune": ([I, I], I),
        "EPSGB300ServerCreate": ([D, I, I, PP], I),
        "EPSGB300ServerSubmit": ([P, P], I),
        "EPSGB300ServerWait": ([P, P, D, ctypes.POINTER(I)], I),
        "EPSGB300ServerGetStats": ([P, P], I),
        "EPSGB300ServerDestroy": ([PP], I),
        "EPSGB300ServerCancel": ([P], I),
        "EPSGB300SetTimeLimit": ([P, D], I),
        "EPSGB300SetGraphCapture": ([P, I], I),
        "EPSSetDeflationSpace": ([P, I, P], I),
        "EPSGB300SetRestartMethod": ([P, I], I),
        "EPSGB300SetGSMethod": ([P, I], I),
        "EPSGB300BatchGetTuning": ([ctypes.POINTER(I), I], I),
        "EPSGB300BatchSetTuning": ([ctypes.POINTER(I), I], I),
        "EPSGB300GetStats": ([P, P], I),
        "EPSGB300OrthogonalityError": ([P, P], I),
        "EPSGB300GetDeviceEigenvectors": ([P, PP, P], I),
        "EPSGB300SetProfiling": ([P, I], I),
        "EPSGB300GetProfile": ([P, I, P, P, P], I),
        "EPSSetExtraction": ([P, I], I),
        "EPSGetExtraction": ([P, P], I),
        "EPSSetTarget": ([P, D], I),
        "EPSSetConvergenceTest": ([P, I], I),
        "EPSGetConvergenceTest": ([P, P], I),
        "EPSSetPurify": ([P, I], I),
        "EPSGetTarget": ([P, P], I),
        "PetscViewerBinaryOpen": ([I, ctypes.c_char_p, I, PP], I),
        "PetscViewerDestroy": ([PP], I),
        "MatCreate": ([I, PP], I),
        "MatLoad": ([P, P], I),
        "MatView": ([P, P], I),
        "PetscViewerASCIIOpen": ([I, ctypes.c_char_p, PP], I),
        "PetscViewerPushFormat": ([P, I], I),
        "PetscViewerPopFormat": ([P], I),
        "EPSErrorView": ([P, I, P], I),
        "SlepcInitialize": ([ctypes.POINTER(I), ctypes.POINTER(ctypes.POINTER(ctypes.c_char_p)), P, P], I),
        "EPSSetFromOptions": ([P], I),
        "PetscObjectSetName": ([P, ctypes.c_char_p], I),
        "EPSMonitorSet": ([P, P, P, P], I),
        "EPSMonitorCancel": ([P], I),
        "EPSConvergedReasonView": ([P, P], I),
        "EPSValuesView": ([P, P], I),
        "EPSView": ([P, P], I),
        "EPSSetOptionsPrefix": ([P, ctypes.c_char_p], I),
        "EPSAppendOptionsPrefix": ([P, ctypes.c_char_p], I),
        "EPSGetOptionsPrefix": ([P, ctypes.POINTER(ctypes.c_char_p)], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


_argv_keep = None


def initialize(argv):
    """SlepcInitialize with this argument list (argv[0] is the program name); EPS.setFromOptions reads it."""
    global _argv_keep
    arr = (ctypes.c_char_p * (len(argv) + 1))(*[a.encode() for a in argv], None)
    argc = ctypes.c_int(len(argv))
    parr = ctypes.cast(arr, ctypes.POINTER(ctypes.c_char_p))
    _argv_keep = (arr, argc, parr)
    _check(load().SlepcInitialize(ctypes.byref(argc), ctypes.byref(parr), None, None), "SlepcInitialize")


# EPSMonitorFn: (eps, its, nconv, eigr, eigi, errest, nest, ctx) -> PetscErrorCode
MONITOR_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p)


def _check(code, where):
    if code:
        msg = load().PetscGB300LastError().decode(errors="replace")
        raise SlepcError(code, where, msg)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Vec:
    """A host vector wrapping a numpy float64 array (VecCreateSeqWithArray)."""

    def __init__(self, array):
        self.array = np.ascontiguousarray(array, dtype=np.float64)
        self.handle = ctypes.c_void_p()
        _check(load().VecCreateSeqWithArray(0, 1, self.array.size, _ptr(self.array), ctypes.byref(self.handle)),
               "VecCreateSeqWithArray")

    def destroy(self):
        if self.handle:
            load().VecDestroy(ctypes.byref(self.handle))

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Mat:
    """CSR matrix over caller-owned arrays (MatCreateSeqAIJWithArrays); the arrays are kept alive here."""

    def __init__(self, rowptr, colidx, vals, ncols=None):
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.colidx = np.ascontiguousarray(colidx, dtype=np.int32)
        self.vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.m = self.rowptr.size - 1
        self.n = self.m if ncols is None else int(ncols)
        self.handle = ctypes.c_void_p()
        _check(load().MatCreateSeqAIJWithArrays(0, self.m, self.n, _ptr(self.rowptr), _ptr(self.colidx),
                                                _ptr(self.vals), ctypes.byref(self.handle)),
               "MatCreateSeqAIJWithArrays")

    @classmethod
    def createAIJ(cls, csr):
        return cls(*csr)

    @classmethod
    def load(cls, path):
        """MatLoad from a PETSc binary file (PetscViewerBinaryOpen + MatCreate + MatLoad); the library owns the
        arrays, and rowptr/colidx/vals are copies of them."""
        lib = load()
        viewer, h = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib.PetscViewerBinaryOpen(0, os.fsencode(path), 0, ctypes.byref(viewer)), "PetscViewerBinaryOpen")
        try:
            _check(lib.MatCreate(0, ctypes.byref(h)), "MatCreate")
            rc = lib.MatLoad(h, viewer)
            if rc:
                lib.MatDestroy(ctypes.byref(h))
                _check(rc, "MatLoad")
        finally:
            lib.PetscViewerDestroy(ctypes.byref(viewer))
        m = ctypes.c_int()
        ia, ja = ctypes.POINTER(ctypes.c_int)(), ctypes.POINTER(ctypes.c_int)()
        aa = ctypes.POINTER(ctypes.c_double)()
        done = ctypes.c_int()
        _check(lib.MatGetRowIJ(h, 0, 0, 0, ctypes.byref(m), ctypes.byref(ia), ctypes.byref(ja), ctypes.byref(done)),
               "MatGetRowIJ")
        _check(lib.MatSeqAIJGetArrayRead(h, ctypes.byref(aa)), "MatSeqAIJGetArrayRead")
        obj = cls.__new__(cls)
        obj.handle = h
        obj.m = m.value
        rows, cols = ctypes.c_int(), ctypes.c_int()
        _check(lib.MatGetSize(h, ctypes.byref(rows), ctypes.byref(cols)), "MatGetSize")
        obj.n = cols.value
        obj.rowptr = np.ctypeslib.as_array(ia, (obj.m + 1,)).copy()
        nnz = int(obj.rowptr[-1])
        obj.colidx = np.ctypeslib.as_array(ja, (nnz,)).copy() if nnz else np.zeros(0, np.int32)
        obj.vals = np.ctypeslib.as_array(aa, (nnz,)).copy() if nnz else np.zeros(0)
        return obj

    def save(self, path):
        """MatView into a PETSc binary file (the format MatLoad and PETSc read)."""
        lib = load()
        viewer = ctypes.c_void_p()
        _check(lib.PetscViewerBinaryOpen(0, os.fsencode(path), 1, ctypes.byref(viewer)), "PetscViewerBinaryOpen")
        try:
            _check(lib.MatView(self.handle, viewer), "MatView")
        finally:
            _check(lib.PetscViewerDestroy(ctypes.byref(viewer)), "PetscViewerDestroy")

    def mult(self, x):
        y = np.zeros(self.m)
        vx, vy = Vec(x), Vec(y)
        _check(load().MatMult(self.handle, vx.handle, vy.handle), "MatMult")
        return vy.array.copy()

    def destroy(self):
        if self.handle:
            load().MatDestroy(ctypes.byref(self.handle))

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class EPS:
    """Eigenvalue problem solver (EPSKRYLOVSCHUR), mirroring slepc4py.SLEPc.EPS."""

    class ProblemType:
        HEP = 1
        GHEP = 2
        NHEP = 3
        GNHEP = 4

    class Conv:
        ABS = 0
        REL = 1
        NORM = 2

    class Which:
        LARGEST_MAGNITUDE = 1
        SMALLEST_MAGNITUDE = 2
        LARGEST_REAL = 3
        SMALLEST_REAL = 4
        LARGEST_IMAGINARY = 5
        SMALLEST_IMAGINARY = 6

    class ErrorType:
        ABSOLUTE = 0
        RELATIVE = 1
        BACKWARD = 2

    class ConvergedReason:
        CONVERGED_TOL = 1
        DIVERGED_ITS = -1
        DIVERGED_BREAKDOWN = -2
        CONVERGED_ITERATING = 0

    WHICH_NAMES = {"LM": 1, "SM": 2, "LR": 3, "SR": 4, "LI": 5, "SI": 6, "TM": 7, "TR": 8}

    class Extraction:
        RITZ = 0
        HARMONIC = 1

    def __init__(self):
        self.handle = ctypes.c_void_p()
        self._A = None
        self._v0 = None

    def create(self, comm=None):
        _check(load().EPSCreate(0, ctypes.byref(self.handle)), "EPSCreate")
        return self

    def destroy(self):
        if self.handle:
            load().EPSDestroy(ctypes.byref(self.handle))
        return self

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def setType(self, t="krylovschur"):
        _check(load().EPSSetType(self.handle, t.encode()), "EPSSetType")

    def setOperators(self, A, B=None):
        """A, and B for a generalised problem A x = k B x (B diagonal on this path)."""
        self._A = A
        self._B = B
        _check(load().EPSSetOperators(self.handle, A.handle, B.handle if B is not None else None), "EPSSetOperators")

    def setConvergenceTest(self, conv):
        if isinstance(conv, str):
            conv = {"abs": 0, "rel": 1, "norm": 2}[conv]
        _check(load().EPSSetConvergenceTest(self.handle, int(conv)), "EPSSetConvergenceTest")

    def getConvergenceTest(self):
        v = ctypes.c_int()
        _check(load().EPSGetConvergenceTest(self.handle, ctypes.byref(v)), "EPSGetConvergenceTest")
        return v.value

    def setPurify(self, purify=True):
        _check(load().EPSSetPurify(self.handle, int(bool(purify))), "EPSSetPurify")

    def setProblemType(self, ptype):
        _check(load().EPSSetProblemType(self.handle, int(ptype)), "EPSSetProblemType")

    def setDimensions(self, nev=None, ncv=None, mpd=None):
        cur = -2
        _check(load().EPSSetDimensions(self.handle, cur if nev is None else int(nev), cur if ncv is None else int(ncv),
                                       cur if mpd is None else int(mpd)), "EPSSetDimensions")

    def getDimensions(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(load().EPSGetDimensions(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "EPSGetDimensions")
        return a.value, b.value, c.value

    def setTolerances(self, tol=None, max_it=None):
        _check(load().EPSSetTolerances(self.handle, -2.0 if tol is None else float(tol),
                                       -2 if max_it is None else int(max_it)), "EPSSetTolerances")

    def getTolerances(self):
        t, m = ctypes.c_double(), ctypes.c_int()
        _check(load().EPSGetTolerances(self.handle, ctypes.byref(t), ctypes.byref(m)), "EPSGetTolerances")
        return t.value, m.value

    def setWhichEigenpairs(self, which):
        if isinstance(which, str):
            which = self.WHICH_NAMES[which]
        _check(load().EPSSetWhichEigenpairs(self.handle, int(which)), "EPSSetWhichEigenpairs")

    def setFromOptions(self):
        _check(load().EPSSetFromOptions(self.handle), "EPSSetFromOptions")

    def setOptionsPrefix(self, prefix):
        _check(load().EPSSetOptionsPrefix(self.handle, prefix.encode() if prefix else None), "EPSSetOptionsPrefix")

    def appendOptionsPrefix(self, prefix):
        _check(load().EPSAppendOptionsPrefix(self.handle, prefix.encode()), "EPSAppendOptionsPrefix")

    def getOptionsPrefix(self):
        v = ctypes.c_char_p()
        _check(load().EPSGetOptionsPrefix(self.handle, ctypes.byref(v)), "EPSGetOptionsPrefix")
        return v.value.decode() if v.value else None

    def setName(self, name):
        """PetscObjectSetName: the name MATLAB-format reports print."""
        _check(load().PetscObjectSetName(self.handle, name.encode()), "PetscObjectSetName")

    def monitorSet(self, fn):
        """EPSMonitorSet with a Python callable fn(its, nconv, eigr, eigi, errest) called after every restart."""
        def _c(_eps, its, nconv, er, ei, es, nest, _ctx):
            try:
                fn(its, nconv, np.ctypeslib.as_array(er, (nest,)).copy(), np.ctypeslib.as_array(ei, (nest,)).copy(),
                   np.ctypeslib.as_array(es, (nest,)).copy())
                return 0
            except Exception:  # a failing monitor aborts the solve with PETSC_ERR_USER
                return 83
        cb = MONITOR_FN(_c)
        self._monitors = getattr(self, "_monitors", []) + [cb]
        _check(load().EPSMonitorSet(self.handle, ctypes.cast(cb, ctypes.c_void_p), None, None), "EPSMonitorSet")

    def monitorCancel(self):
        _check(load().EPSMonitorCancel(self.handle), "EPSMonitorCancel")
        self._monitors = []

    def setInitialSpace(self, space):
        if space is None or (isinstance(space, (list, tuple)) and len(space) == 0):
            _check(load().EPSSetInitialSpace(self.handle, 0, None), "EPSSetInitialSpace")
            return
        vecs = list(space) if isinstance(space, (list, tuple)) else [space]
        vecs = [x if isinstance(x, Vec) else Vec(x) for x in vecs]
        self._v0 = vecs
        arr = (ctypes.c_void_p * len(vecs))(*[x.handle.value for x in vecs])
        _check(load().EPSSetInitialSpace(self.handle, len(vecs), arr), "EPSSetInitialSpace")

    def setKrylovSchurRestart(self, keep):
        _check(load().EPSKrylovSchurSetRestart(self.handle, float(keep)), "EPSKrylovSchurSetRestart")

    def setExtraction(self, extraction):
        """'ritz' or 'harmonic' (or EPS.Extraction.*): harmonic Rayleigh-Ritz for eigenvalues near the target."""
        if isinstance(extraction, str):
            extraction = {"ritz": 0, "harmonic": 1}[extraction]
        _check(load().EPSSetExtraction(self.handle, int(extraction)), "EPSSetExtraction")

    def getExtraction(self):
        v = ctypes.c_int()
        _check(load().EPSGetExtraction(self.handle, ctypes.byref(v)), "EPSGetExtraction")
        return v.value

    def setTarget(self, target):
        _check(load().EPSSetTarget(self.handle, ctypes.c_double(float(target))), "EPSSetTarget")

    def getTarget(self):
        v = ctypes.c_double()
        _check(load().EPSGetTarget(self.handle, ctypes.byref(v)), "EPSGetTarget")
        return v.value

    def setKrylovSchurLocking(self, lock):
        _check(load().EPSKrylovSchurSetLocking(self.handle, int(bool(lock))), "EPSKrylovSchurSetLocking")

    def setArithmetic(self, arith):
        """'pair' (pair storage, error-free FP32-pair arithmetic), 'f64' (IEEE FP64 FMA) or 'f32' (the precision
        form: FP32 values and basis with pair accumulation, FP64 recheck and refinement sweep)."""
        code = {"pair": 0, "f64": 1, "f32": 2}[arith]
        _check(load().EPSGB300SetArithmetic(self.handle, code), "EPSGB300SetArithmetic")

    RESTART_METHODS = {"tensor": 0, "pair": 1, "mma_sync": 2, "tcgen05": 3}

    def setRestartMethod(self, method):
        """'tensor' (bf16 tensor cores with an error-free split, default), 'pair' (CUDA-core pair arithmetic), or the
        tensor-core kernel explicitly: 'mma_sync' or 'tcgen05' (bit-identical results)."""
        _check(load().EPSGB300SetRestartMethod(self.handle, self.RESTART_METHODS[method]), "EPSGB300SetRestartMethod")

    GS_METHODS = {"tensor": 0, "fma": 1, "integer": 2, "auto": 3}

    def setGSMethod(self, method):
        """'auto' (the default: 'integer' unless the factorisation segments replay from CUDA graphs, then 'fma'),
        'integer' (exact products on the integer pipes), 'fma' (IEEE FP64 FMA) or 'tensor' (exact slice products on
        the tensor cores) for the Gram-Schmidt pair of IEEE-double storage (EPSGB300SetGSMethod)."""
        _check(load().EPSGB300SetGSMethod(self.handle, self.GS_METHODS[method]), "EPSGB300SetGSMethod")

    def setTimeLimit(self, seconds):
        """Wall-time budget of EPSSolve (checked after each restart; 0 = none)."""
        _check(load().EPSGB300SetTimeLimit(self.handle, float(seconds)), "EPSGB300SetTimeLimit")

    def setDeflationSpace(self, vectors):
        """EPSSetDeflationSpace: the eigenvectors sought are orthogonal to the span of these (length-n arrays); the
        vectors are copied."""
        vs = [Vec(np.ascontiguousarray(v, dtype=np.float64)) for v in vectors]
        arr = (ctypes.c_void_p * max(1, len(vs)))(*[v.handle.value for v in vs])
        _check(load().EPSSetDeflationSpace(self.handle, len(vs), arr), "EPSSetDeflationSpace")

    def setGraphCapture(self, mode):
        """Factorisation segments as CUDA graphs: -1 auto (n <= 262144), 0 off, 1 on (EPSGB300SetGraphCapture)."""
        _check(load().EPSGB300SetGraphCapture(self.handle, int(mode)), "EPSGB300SetGraphCapture")

    def setProjectedSolver(self, method):
        """'auto' (default: 'refined' until a restart falls back, then 'qr'), 'qr' (FP64 QL) or
        'refined' (FP32 QL + FP64 refinement with a checked fallback to 'qr') for the symmetric projected problem."""
        code = {"refined": 0, "qr": 1, "auto": 2}[method]
        _check(load().EPSGB300SetProjectedSolver(self.handle, code), "EPSGB300SetProjectedSolver")

    def setUp(self):
        _check(load().EPSSetUp(self.handle), "EPSSetUp")

    def solve(self):
        _check(load().EPSSolve(self.handle), "EPSSolve")

    def getConverged(self):
        v = ctypes.c_int()
        _check(load().EPSGetConverged(self.handle, ctypes.byref(v)), "EPSGetConverged")
        return v.value

    def getConvergedReason(self):
        v = ctypes.c_int()
        _check(load().EPSGetConvergedReason(self.handle, ctypes.byref(v)), "EPSGetConvergedReason")
        return v.value

    def getIterationNumber(self):
        v = ctypes.c_int()
        _check(load().EPSGetIterationNumber(self.handle, ctypes.byref(v)), "EPSGetIterationNumber")
        return v.value

    def getEigenvalue(self, i):
        re, im = ctypes.c_double(), ctypes.c_double()
        _check(load().EPSGetEigenvalue(self.handle, int(i), ctypes.byref(re), ctypes.byref(im)), "EPSGetEigenvalue")
        return complex(re.value, im.value) if im.value != 0.0 else re.value

    def getEigenpair(self, i, Vr=None, Vi=None):
        """Returns the eigenvalue; fills the numpy arrays / Vec objects Vr, Vi (length n) when given."""
        re, im = ctypes.c_double(), ctypes.c_double()
        vr = Vr if (Vr is None or isinstance(Vr, Vec)) else Vec(Vr)
        vi = Vi if (Vi is None or isinstance(Vi, Vec)) else Vec(Vi)
        _check(load().EPSGetEigenpair(self.handle, int(i), ctypes.byref(re), ctypes.byref(im),
                                      vr.handle if vr is not None else None, vi.handle if vi is not None else None),
               "EPSGetEigenpair")
        if Vr is not None and not isinstance(Vr, Vec):
            Vr[...] = vr.array
        if Vi is not None and not isinstance(Vi, Vec):
            Vi[...] = vi.array
        return complex(re.value, im.value) if im.value != 0.0 else re.value

    def getErrorEstimate(self, i):
        v = ctypes.c_double()
        _check(load().EPSGetErrorEstimate(self.handle, int(i), ctypes.byref(v)), "EPSGetErrorEstimate")
        return v.value

    def computeError(self, i, etype=ErrorType.RELATIVE):
        v = ctypes.c_double()
        _check(load().EPSComputeError(self.handle, int(i), int(etype), ctypes.byref(v)), "EPSComputeError")
        return v.value

    # text reports through an ASCII viewer (petsc4py: EPS.errorView / valuesView / convergedReasonView).  With
    # path=None the text is returned (written through a temporary ASCII viewer); otherwise it goes to that file, or
    # to the process's stdout for path="stdout".  detail=True pushes PETSC_VIEWER_ASCII_INFO_DETAIL.
    def _view(self, fn, args, path, detail):
        import tempfile
        lib = load()
        tmp = None
        if path is None:
            fd, tmp = tempfile.mkstemp(suffix=".txt")
            os.close(fd)
        viewer = ctypes.c_void_p()
        _check(lib.PetscViewerASCIIOpen(0, os.fsencode(tmp or path), ctypes.byref(viewer)), "PetscViewerASCIIOpen")
        try:
            if detail:
                _check(lib.PetscViewerPushFormat(viewer, 5), "PetscViewerPushFormat")
            _check(getattr(lib, fn)(self.handle, *args, viewer), fn)
        finally:
            _check(lib.PetscViewerDestroy(ctypes.byref(viewer)), "PetscViewerDestroy")
        if tmp is None:
            return None
        with open(tmp) as f:
            text = f.read()
        os.unlink(tmp)
        return text

    def errorView(self, etype=ErrorType.RELATIVE, path=None, detail=False):
        return self._view("EPSErrorView", (int(etype),), path, detail)

    def convergedReasonView(self, path=None):
        return self._view("EPSConvergedReasonView", (), path, False)

    def valuesView(self, path=None):
        return self._view("EPSValuesView", (), path, False)

    def view(self, path=None):
        """EPSView: the solver configuration (before EPSSetUp the values set, after it the values in use)."""
        return self._view("EPSView", (), path, False)

    def getStats(self):
        buf = (ctypes.c_char * 96)()
        _check(load().EPSGB300GetStats(self.handle, buf), "EPSGB300GetStats")
        steps, restarts = np.frombuffer(bytes(buf[:16]), dtype=np.int64)
        solve_s, bytes_moved, setup_s = np.frombuffer(bytes(buf[16:40]), dtype=np.float64)
        launches = np.frombuffer(bytes(buf[40:48]), dtype=np.int64)[0]
        dev_ms = np.frombuffer(bytes(buf[48:56]), dtype=np.float64)[0]
        psteps, prestarts, dsfb, graphs, gs_exact = np.frombuffer(bytes(buf[56:96]), dtype=np.int64)
        return {"krylov_steps": int(steps), "restarts": int(restarts), "solve_seconds": float(solve_s),
                "bytes_moved": float(bytes_moved), "setup_seconds": float(setup_s), "kernel_launches": int(launches),
                "solve_device_ms": float(dev_ms), "precision_steps": int(psteps),
                "precision_restarts": int(prestarts), "ds_fallbacks": int(dsfb), "graph_segments": int(graphs),
                "gs_exact": int(gs_exact)}

    KERNEL_CLASSES = ("spmv", "gs_dot", "gs_update", "restart", "ds")

    def setProfiling(self, on=True):
        _check(load().EPSGB300SetProfiling(self.handle, int(bool(on))), "EPSGB300SetProfiling")

    def getProfile(self):
        """{class: (device ms, algorithmic bytes, launches)} accumulated since setProfiling(True)."""
        out = {}
        for c, name in enumerate(self.KERNEL_CLASSES):
            ms, by, nl = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
            _check(load().EPSGB300GetProfile(self.handle, c, ctypes.byref(ms), ctypes.byref(by), ctypes.byref(nl)),
                   "EPSGB300GetProfile")
            out[name] = (ms.value, by.value, nl.value)
        return out

    def getDeviceEigenvectors(self):
        """(device address, leading dimension) of the FP64 eigenvector array (EPSGB300GetDeviceEigenvectors)."""
        p, ld = ctypes.c_void_p(), ctypes.c_int()
        _check(load().EPSGB300GetDeviceEigenvectors(self.handle, ctypes.byref(p), ctypes.byref(ld)),
               "EPSGB300GetDeviceEigenvectors")
        return p.value, ld.value

    def copyDeviceEigenvectors(self):
        """The device eigenvector array copied to the host (n x nconv), one cudaMemcpy of the columns."""
        ptr, ld = self.getDeviceEigenvectors()
        m = self.getConverged()
        n = self._A.m
        out = np.empty((m, ld))
        if m:
            rt = ctypes.CDLL("libcudart.so")
            rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            err = rt.cudaMemcpy(out.ctypes.data, ctypes.c_void_p(ptr), out.nbytes, 2)  # cudaMemcpyDeviceToHost
            if err != 0:
                raise SlepcError(err, "cudaMemcpy", "device eigenvector copy failed")
        return np.ascontiguousarray(out[:, :n].T)

    def orthogonalityError(self):
        v = ctypes.c_double()
        _check(load().EPSGB300OrthogonalityError(self.handle, ctypes.byref(v)), "EPSGB300OrthogonalityError")
        return v.value


def solve_batch(eps_list):
    """EPSGB300SolveBatch over configured EPS objects (the batched engine); results are read from each EPS."""
    arr = (ctypes.c_void_p * len(eps_list))(*[e.handle for e in eps_list])
    _check(load().EPSGB300SolveBatch(len(eps_list), arr), "EPSGB300SolveBatch")


BATCH_BUCKETS = 14


class _ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_longlong) for k in
                ("submitted", "completed", "failed", "queued", "live", "max_live", "cycles")] + \
               [("bytes_in_use", ctypes.c_double), ("peak_bytes", ctypes.c_double)]


class Server:
    """EPSGB300Server: continuous-batching request loop over the batched engine (its own host thread)."""

    def __init__(self, hbm_budget_bytes, max_requests=4096, max_ncv=72):
        h = ctypes.c_void_p()
        _check(load().EPSGB300ServerCreate(float(hbm_budget_bytes), int(max_requests), int(max_ncv),
                                           ctypes.byref(h)), "EPSGB300ServerCreate")
        self.handle = h
        self._inflight = {}

    def submit(self, eps):
        _check(load().EPSGB300ServerSubmit(self.handle, eps.handle), "EPSGB300ServerSubmit")
        self._inflight[eps.handle.value] = eps

    def wait(self, eps, timeout=-1.0):
        done = ctypes.c_int(0)
        try:
            _check(load().EPSGB300ServerWait(self.handle, eps.handle, float(timeout), ctypes.byref(done)),
                   "EPSGB300ServerWait")
        finally:
            if done.value:
                self._inflight.pop(eps.handle.value, None)
        return bool(done.value)

    def cancel(self):
        _check(load().EPSGB300ServerCancel(self.handle), "EPSGB300ServerCancel")

    def stats(self):
        st = _ServerStats()
        _check(load().EPSGB300ServerGetStats(self.handle, ctypes.byref(st)), "EPSGB300ServerGetStats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def destroy(self):
        if self.handle:
            h = self.handle
            self.handle = None
            _check(load().EPSGB300ServerDestroy(ctypes.byref(h)), "EPSGB300ServerDestroy")


def batch_tune(first_bucket=1, last_bucket=7):
    """Measure the batched engine's tiles per virtual block for size buckets first..last; returns the table."""
    _check(load().EPSGB300BatchTune(first_bucket, last_bucket), "EPSGB300BatchTune")
    return batch_get_tuning()


def batch_get_tuning():
    arr = (ctypes.c_int * BATCH_BUCKETS)()
    _check(load().EPSGB300BatchGetTuning(arr, BATCH_BUCKETS), "EPSGB300BatchGetTuning")
    return list(arr)


def batch_set_tuning(tiles):
    arr = (ctypes.c_int * BATCH_BUCKETS)(*tiles)
    _check(load().EPSGB300BatchSetTuning(arr, len(tiles)), "EPSGB300BatchSetTuning")


def solve(csr, *, hermitian=True, which="LM", nev=1, ncv=None, mpd=None, tol=None, max_it=None, v0=None,
          arith="pair", vectors=True, ds=None, lock=None, restart=None, harmonic=False, target=None, B=None,
          conv=None, purify=None, gs=None, keep=None, deflation=None):
    """One-call convenience: returns dict(eigr, eigi, X, nconv, its, reason, errors, stats).  B (CSR arrays of a
    diagonal matrix) makes the problem generalised: EPS_GHEP when hermitian, else EPS_GNHEP."""
    A = Mat(*csr)
    Bm = Mat(*B) if B is not None else None
    eps = EPS().create()
    eps.setOperators(A, Bm)
    if Bm is None:
        eps.setProblemType(EPS.ProblemType.HEP if hermitian else EPS.ProblemType.NHEP)
    else:
        eps.setProblemType(EPS.ProblemType.GHEP if hermitian else EPS.ProblemType.GNHEP)
    if conv is not None:
        eps.setConvergenceTest(conv)
    if purify is not None:
        eps.setPurify(purify)
    eps.setDimensions(nev, ncv if ncv else -1, mpd if mpd else -1)
    eps.setTolerances(tol if tol else -1.0, max_it if max_it else -1)
    eps.setWhichEigenpairs(which)
    eps.setArithmetic(arith)
    if target is not None:
        eps.setTarget(target)
    if harmonic:
        eps.setExtraction("harmonic")
    if ds is not None:
        eps.setProjectedSolver(ds)
    if restart is not None:
        eps.setRestartMethod(restart)
    if gs is not None:
        eps.setGSMethod(gs)
    if lock is not None:
        eps.setKrylovSchurLocking(lock)
    if keep is not None:
        eps.setKrylovSchurRestart(keep)
    if deflation is not None:
        eps.setDeflationSpace(list(np.asarray(deflation, dtype=np.float64).reshape(A.m, -1).T))
    if v0 is not None:
        eps.setInitialSpace(v0)
    eps.solve()
    nconv = eps.getConverged()
    n = A.m
    eigr = np.zeros(nconv)
    eigi = np.zeros(nconv)
    X = np.zeros((n, nconv)) if vectors else None
    for i in range(nconv):
        xr = np.zeros(n)
        lam = eps.getEigenpair(i, xr if vectors else None)
        eigr[i] = lam.real if isinstance(lam, complex) else lam
        eigi[i] = lam.imag if isinstance(lam, complex) else 0.0
        if vectors:
            X[:, i] = xr
    out = {"eigr": eigr, "eigi": eigi, "X": X, "nconv": nconv, "its": eps.getIterationNumber(),
           "reason": eps.getConvergedReason(), "stats": eps.getStats(),
           "errors": np.array([eps.computeError(i) for i in range(nconv)]), "eps": eps, "A": A, "B": Bm}
    return out
