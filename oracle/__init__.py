"""The oracle: a CPU restatement of SLEPc 3.22's Krylov-Schur path (ks_oracle.c), loaded through ctypes.

TEST INFRASTRUCTURE ONLY.  It is what the CUDA path is compared against in the tests, and the timed CPU baseline.
Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and its reference arm) may import it;
the product package slepc_gb300 never does.

``build()`` compiles ``ks_oracle.c`` into ``oracle/_build/libksoracle.so`` with gcc -O3 -fopenmp (portable
flags only: the same source builds on x86_64 and aarch64).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libksoracle.so")

WHICH = {"LM": 1, "SM": 2, "LR": 3, "SR": 4, "LI": 5, "SI": 6, "TM": 7, "TR": 8}
INFO_LEN = 16
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ks_oracle.c")
    os.makedirs(LIB_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-D_POSIX_C_SOURCE=200809L",
               "-o", LIB_PATH + ".tmp", src, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i, d, ull = ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong
        lib.ksor_solve.argtypes = [i, P, P, P, i, i, i, i, i, d, i, d, i, i, P, ull, d, P, i, P, P, P, P, i, d]
        lib.ksor_solve.restype = i
        lib.ksor_solve_gen.argtypes = [i, P, P, P, P, i, i, i, i, i, d, i, d, i, i, P, ull, d, P, i, P, P, P, P, i, d,
                                       i, d, d, i]
        lib.ksor_solve_gen.restype = i
        lib.ksor_solve_genb.argtypes = [i, P, P, P, P, P, P, i, i, i, i, i, d, i, d, i, i, P, ull, d, P, i, P, P, P,
                                        P, i, d, i, d, d, i]
        lib.ksor_solve_genb.restype = i
        lib.ksor_set_monitor.argtypes = [MONITOR_FN, P]
        lib.ksor_set_monitor.restype = None
        lib.ksor_set_deflation.argtypes = [i, P]
        lib.ksor_set_deflation.restype = None
        lib.ksor_spmv.argtypes = [i, P, P, P, P, P, i]
        lib.ksor_spmv.restype = None
        lib.ksor_ds_hep.argtypes = [i, i, i, i, P, P, i, i, i, P, P, P]
        lib.ksor_ds_hep.restype = i
        lib.ksor_ds_nhep.argtypes = [i, i, P, i, i, i, P, P, P, i, P, P]
        lib.ksor_ds_nhep.restype = i
        lib.ksor_schur.argtypes = [i, i, P, P, P, P]
        lib.ksor_schur.restype = i
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Result:
    """Outcome of one oracle solve (fields mirror EPSGetConverged / EPSGetIterationNumber / ...)."""

    def __init__(self, info, eigr, eigi, errest, X, err):
        self.err = err
        self.nconv = int(info[0])
        self.its = int(info[1])
        self.reason = int(info[2])
        self.nsteps = int(info[3])
        self.npasses = int(info[4])
        self.ncv = int(info[5])
        self.mpd = int(info[6])
        self.max_it = int(info[7])
        self.eigr = eigr[: self.nconv].copy()
        self.eigi = eigi[: self.nconv].copy()
        self.errest = errest[: self.nconv].copy()
        self.X = X[:, : self.nconv] if X is not None else None


CONV = {"abs": 0, "rel": 1, "norm": 2}


MONITOR_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                              ctypes.c_void_p)


def solve(rowptr, colidx, vals, *, hermitian=True, which="LM", nev=1, ncv=0, mpd=0, tol=1e-8, max_it=0,
          keep=0.5, lock=True, v0=None, nthreads=1, seed=0x5EED, time_budget=0.0, vectors=True, harmonic=False,
          target=0.0, bdiag=None, conv="rel", purify=True, monitor=None, B=None, deflation=None) -> Result:
    """bdiag: the diagonal of B for A x = k B x (EPS_GHEP when hermitian, else EPS_GNHEP); conv: "rel", "abs" or
    "norm" (EPS_CONV_NORM with the infinity norms of A and of B, or 0 for ||B|| without B, as EPSSetUp leaves it);
    deflation: an n x nds array whose columns span the deflation space (EPSSetDeflationSpace)."""
    lib = load()
    n = len(rowptr) - 1
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colidx = np.ascontiguousarray(colidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    cap = max(ncv if ncv > 0 else 0, nev + 15, 2 * nev, nev + (mpd if mpd > 0 else 0)) + 1
    cap = min(cap, n) if n > 0 else cap
    cap = max(cap, 1)
    info = np.zeros(INFO_LEN, dtype=np.int32)
    eigr = np.zeros(cap)
    eigi = np.zeros(cap)
    errest = np.zeros(cap)
    X = np.asfortranarray(np.zeros((n, cap))) if vectors else None  # column-major n x cap
    v0a = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64)
    bd = None if bdiag is None else np.ascontiguousarray(bdiag, dtype=np.float64)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    nrma = float(np.bincount(rows, weights=np.abs(vals), minlength=n).max()) if conv == "norm" and n else 0.0
    nrmb = float(np.max(np.abs(bd))) if conv == "norm" and bd is not None else 0.0
    if B is not None:
        brp, bci, bva = (np.ascontiguousarray(B[0], np.int32), np.ascontiguousarray(B[1], np.int32),
                         np.ascontiguousarray(B[2], np.float64))
        brows = np.repeat(np.arange(n), np.diff(brp))
        if conv == "norm":
            nrmb = float(np.bincount(brows, weights=np.abs(bva), minlength=n).max())
    cb = None
    if monitor is not None:
        def _mon(its, nconv, er, ei, es, nest, _ctx):
            monitor(its, nconv, [er[i] for i in range(nest)], [ei[i] for i in range(nest)],
                    [es[i] for i in range(nest)], nest)
        cb = MONITOR_FN(_mon)
    lib.ksor_set_monitor(cb if cb is not None else MONITOR_FN(), None)
    W = None if deflation is None else np.asfortranarray(np.asarray(deflation, np.float64).reshape(n, -1))
    lib.ksor_set_deflation(0 if W is None else W.shape[1], _ptr(W))
    if B is None:
        err = lib.ksor_solve_gen(n, _ptr(rowptr), _ptr(colidx), _ptr(vals), _ptr(bd), int(bool(hermitian)),
                                 WHICH[which], int(nev), int(ncv), int(mpd), float(tol), int(max_it), float(keep),
                                 int(bool(lock)), int(nthreads), _ptr(v0a), int(seed), float(time_budget), _ptr(info),
                                 int(cap), _ptr(eigr), _ptr(eigi), _ptr(errest), _ptr(X), int(bool(harmonic)),
                                 float(target), CONV[conv], nrma, nrmb, int(bool(purify)))
    else:
        err = lib.ksor_solve_genb(n, _ptr(rowptr), _ptr(colidx), _ptr(vals), _ptr(brp), _ptr(bci), _ptr(bva),
                                  int(bool(hermitian)), WHICH[which], int(nev), int(ncv), int(mpd), float(tol),
                                  int(max_it), float(keep), int(bool(lock)), int(nthreads), _ptr(v0a), int(seed),
                                  float(time_budget), _ptr(info), int(cap), _ptr(eigr), _ptr(eigi), _ptr(errest),
                                  _ptr(X), int(bool(harmonic)), float(target), CONV[conv], nrma, nrmb,
                                  int(bool(purify)))
    lib.ksor_set_monitor(MONITOR_FN(), None)
    lib.ksor_set_deflation(0, None)
    return Result(info, eigr, eigi, errest, X, err)


def spmv(rowptr, colidx, vals, x, nthreads=1):
    lib = load()
    n = len(rowptr) - 1
    y = np.zeros(n)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib.ksor_spmv(n, _ptr(np.ascontiguousarray(rowptr, np.int32)), _ptr(np.ascontiguousarray(colidx, np.int32)),
                  _ptr(np.ascontiguousarray(vals, np.float64)), _ptr(x), _ptr(y), int(nthreads))
    return y


def ds_hep(n, l, k, d, e, *, ld=None, state_raw=True, which="LM", extrarow=False):
    lib = load()
    ld = n + 2 if ld is None else ld
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    wr = np.zeros(n)
    Q = np.zeros(ld * ld)
    eout = np.zeros(n)
    err = lib.ksor_ds_hep(n, l, k, ld, _ptr(d), _ptr(e), int(state_raw), WHICH[which], int(extrarow), _ptr(wr),
                          _ptr(Q), _ptr(eout))
    return err, wr, Q.reshape(ld, ld).T, eout


def ds_nhep(A, *, ld=None, intermediate=True, which="LM", extrarow=False, vec_index=-1):
    """A: (n or n+1) x n matrix (extra row included when extrarow).  Returns err, wr, wi, T, Q, rnorm, X."""
    lib = load()
    n = A.shape[1]
    ld = n + 2 if ld is None else ld
    Af = np.zeros((ld, ld))
    Af[: A.shape[0], :n] = A
    Af = np.asfortranarray(Af)
    Q = np.asfortranarray(np.zeros((ld, ld)))
    X = np.asfortranarray(np.zeros((ld, ld)))
    wr = np.zeros(n)
    wi = np.zeros(n)
    rnorm = np.zeros(1)
    err = lib.ksor_ds_nhep(n, ld, _ptr(Af), int(intermediate), WHICH[which], int(extrarow), _ptr(wr), _ptr(wi),
                           _ptr(Q), int(vec_index), _ptr(rnorm), _ptr(X))
    return err, wr, wi, Af, Q, float(rnorm[0]), X


def schur(A):
    lib = load()
    n = A.shape[0]
    Af = np.asfortranarray(A.astype(np.float64).copy())
    Q = np.asfortranarray(np.zeros((n, n)))
    wr = np.zeros(n)
    wi = np.zeros(n)
    err = lib.ksor_schur(n, n, _ptr(Af), _ptr(Q), _ptr(wr), _ptr(wi))
    return err, Af, Q, wr, wi
