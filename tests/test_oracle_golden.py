"""The oracle (CPU restatement of SLEPc's Krylov-Schur) pinned against the reference's own expected outputs and
against closed-form spectra / dense LAPACK (numpy, scipy)."""
import json
import os

import numpy as np
import pytest

from slepc_gb300 import matgen

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))
EPS64 = np.finfo(float).eps


def r5(x):
    return [round(float(v), 5) for v in x]


def test_ds_hep_arrow_golden(orc):
    g = G["ds_test3_1"]
    n, l, k = g["n"], g["l"], g["k"]
    d = np.arange(1, n + 1, dtype=float)
    e = np.zeros(n)
    e[l:n - 1] = 1.0
    err, wr, Q, _ = orc.ds_hep(n, l, k, d, e, which="LM")
    assert err == 0
    assert r5(wr) == g["eigenvalues"]
    # same spectrum as the dense arrow matrix
    T = np.diag(d)
    for i in range(l, k):
        T[i, k] = T[k, i] = 1.0
    for i in range(k, n - 1):
        T[i, i + 1] = T[i + 1, i] = 1.0
    assert np.allclose(np.sort(wr), np.sort(np.linalg.eigvalsh(T)), atol=1e-13)


def test_ds_hep_extrarow(orc):
    n, l, k = 9, 2, 5
    d = np.arange(1, n + 1, dtype=float)
    e = np.zeros(n)
    e[l:n - 1] = 1.0
    e[n - 1] = 1.0
    err, wr, Q, eout = orc.ds_hep(n, l, k, d, e, which="LM", extrarow=True)
    assert err == 0
    assert abs(np.sum(eout[l:n] - Q[n - 1, l:n])) < 10 * EPS64


def grcar(n):
    A = np.zeros((n, n))
    for i in range(1, n):
        A[i, i - 1] = -1.0
    for j in range(4):
        for i in range(n - j):
            A[i, i + j] = 1.0
    return A


def test_ds_nhep_golden(orc):
    g = G["ds_test1_1"]
    n = g["n"]
    err, wr, wi, T, Q, rn, X = orc.ds_nhep(grcar(n), which="LM", vec_index=2)
    assert err == 0
    got = [[round(a, 5), round(abs(b), 5)] for a, b in zip(wr, wi)]
    assert got == g["eigenvalues_abs_imag"]
    assert round(rn, 3) == g["rnorm_3rd"]
    assert round(np.hypot(np.linalg.norm(X[:n, 0]), np.linalg.norm(X[:n, 1])), 3) == g["norm_1st"]
    # Schur relation A Q = Q T
    A = grcar(n)
    assert np.abs(A @ Q[:n, :n] - Q[:n, :n] @ T[:n, :n]).max() < 1e-13


def test_ex2_golden(orc):
    g = G["ex2_1"]
    nx, ny = g["grid"]
    csr = matgen.laplacian_2d(nx, ny)
    r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], ncv=g["ncv"], tol=1e-8,
                  v0=matgen.start_vector(nx * ny, 1))
    assert r.err == 0 and r.reason == 1 and r.nconv >= g["nev"]
    assert r5(r.eigr[: g["nev"]]) == g["eigenvalues"]


@pytest.mark.parametrize("key", ["test2_1", "test2_3"])
def test_test2_golden(orc, key):
    g = G[key]
    csr = matgen.laplacian_1d(g["n"])
    tol = max(1000 * EPS64, 1e-9)
    for which, name in (("LR", "largest"), ("SR", "smallest")):
        for lock in (True, False):
            r = orc.solve(*csr, hermitian=True, which=which, nev=g["nev"], tol=tol, lock=lock,
                          v0=matgen.start_vector(g["n"], 1))
            assert r.err == 0 and r.reason == 1
            assert r5(r.eigr[: g["nev"]]) == g[name]


def test_ex9_golden(orc):
    g = G["ex9_1"]
    csr = matgen.brusselator(g["N"])
    r = orc.solve(*csr, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-8,
                  v0=matgen.start_vector(2 * g["N"], 1))
    assert r.err == 0 and r.reason == 1
    assert [[round(a, 5), round(b, 5)] for a, b in zip(r.eigr[:4], r.eigi[:4])] == g["eigenvalues"]


def test_convdiff_analytic(orc):
    N, Pe = 40, 10.0
    csr = matgen.convection_diffusion_2d(N, Pe)
    r = orc.solve(*csr, hermitian=False, which="LR", nev=10, ncv=40, tol=1e-12, v0=matgen.start_vector(N * N, 3))
    assert r.err == 0 and r.reason == 1
    ex = matgen.convdiff_eigenvalues(N, Pe)
    for lam in r.eigr:
        assert np.min(np.abs(ex - lam)) / abs(lam) < 1e-10
    assert np.max(np.abs(r.eigi)) == 0.0


def test_lap3d_analytic_and_orthogonality(orc):
    m = 12
    csr = matgen.laplacian_3d(m)
    r = orc.solve(*csr, hermitian=True, which="LR", nev=20, ncv=48, tol=1e-10, v0=matgen.start_vector(m ** 3, 2))
    assert r.err == 0 and r.reason == 1
    ex = matgen.laplacian_eigenvalues([m, m, m])
    assert max(np.min(np.abs(ex - l)) / abs(l) for l in r.eigr) < 1e-12
    assert np.abs(r.X.T @ r.X - np.eye(r.nconv)).max() < 1e-12
    A = matgen.csr_to_dense(*csr)
    res = [np.linalg.norm(A @ r.X[:, i] - r.eigr[i] * r.X[:, i]) / (np.linalg.norm(A, 2) * abs(r.eigr[i]))
           for i in range(r.nconv)]
    assert max(res) < 1e-10


def test_dense_nhep_against_numpy(orc):
    rng = np.random.default_rng(7)
    for n in (5, 17, 40):
        A = rng.standard_normal((n, n))
        err, T, Q, wr, wi = orc.schur(A)
        assert err == 0
        assert np.abs(Q.T @ Q - np.eye(n)).max() < 1e-13
        assert np.abs(A @ Q - Q @ T).max() < 1e-12 * np.abs(A).max() * n
        ev = np.linalg.eigvals(A)
        got = wr + 1j * wi
        for z in got:
            assert np.min(np.abs(ev - z)) < 1e-10 * max(1, abs(z))


def test_zero_start_vector_is_an_error(orc):
    csr = matgen.laplacian_1d(40)
    r = orc.solve(*csr, hermitian=True, which="LM", nev=2, v0=np.zeros(40))
    assert r.err != 0


def test_spmv(orc):
    csr = matgen.convection_diffusion_2d(20, 5.0)
    x = matgen.start_vector(400, 9)
    A = matgen.csr_to_dense(*csr)
    assert np.allclose(orc.spmv(*csr, x), A @ x, rtol=0, atol=1e-14)


@pytest.mark.parametrize("lock", [True, False])
def test_test2_interior_harmonic_golden(orc, lock):
    """src/eps/tests/test2.c third solve: EPS_TARGET_MAGNITUDE, target 2.1, EPSSetExtraction(EPS_HARMONIC)."""
    g = G["test2_1"]
    csr = matgen.laplacian_1d(g["n"])
    r = orc.solve(*csr, hermitian=True, which="TM", nev=g["nev"], tol=g["tol"], v0=matgen.start_vector(g["n"], 1),
                  harmonic=True, target=g["target"], lock=lock)
    assert r.err == 0 and r.reason == 1
    assert [round(v, 5) for v in r.eigr[:4]] == g["interior"]


def test_harmonic_interior_analytic(orc):
    n, tgt = 200, 2.1
    csr = matgen.laplacian_1d(n)
    r = orc.solve(*csr, hermitian=True, which="TM", nev=4, ncv=24, tol=1e-10, v0=matgen.start_vector(n, 1),
                  harmonic=True, target=tgt)
    assert r.err == 0 and r.reason == 1
    ex = 2 - 2 * np.cos(np.arange(1, n + 1) * np.pi / (n + 1))
    want = ex[np.argsort(np.abs(ex - tgt))][:4]
    assert np.max(np.abs(np.asarray(r.eigr[:4]) - want) / want) < 1e-12


def test_ghep_test1_golden(orc):
    """test1.c: A x = k B x with the 2-D Laplacian and B = diag(2/log(i+2)), EPS_GHEP, EPS_CONV_NORM, tol 1e-10:
    the digits of test1_1.out, B-orthonormal purified eigenvectors, and scipy's dense generalised solver."""
    import scipy.linalg as sl
    g = G["test1_1"]
    csr = matgen.laplacian_2d(*g["grid"])
    n = g["grid"][0] * g["grid"][1]
    b = matgen.log_mass(n)
    r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"], max_it=g["max_it"],
                  conv=g["conv"], bdiag=b, v0=matgen.start_vector(n, 1))
    assert r.err == 0 and r.reason == 1
    assert r5(r.eigr[:4]) == g["eigenvalues"]
    X = r.X[:, :r.nconv]
    assert np.abs(X.T @ (b[:, None] * X) - np.eye(r.nconv)).max() < 10 * g["tol"]  # test1.c's orthogonality check
    w = np.sort(sl.eigh(matgen.csr_to_dense(*csr), np.diag(b), eigvals_only=True))[::-1]
    for lam in r.eigr[:r.nconv]:
        assert np.min(np.abs(w - lam)) / abs(lam) < 1e-11


def test_gnhep_against_scipy(orc):
    """EPS_GNHEP with a diagonal B: B^-1 A with the Euclidean inner product, against scipy.linalg.eig(A, B)."""
    import scipy.linalg as sl
    N = 20
    csr = matgen.convection_diffusion_2d(N, 2.0)
    n = N * N
    b = 1.0 + matgen.uniform_01(11, n)
    r = orc.solve(*csr, hermitian=False, which="LR", nev=6, tol=1e-11, bdiag=b, v0=matgen.start_vector(n, 2))
    assert r.err == 0 and r.reason == 1
    w = sl.eig(matgen.csr_to_dense(*csr), np.diag(b), right=False)
    for a, c in zip(r.eigr[:r.nconv], r.eigi[:r.nconv]):
        z = complex(a, c)
        assert np.min(np.abs(w - z)) / abs(z) < 1e-10


@pytest.mark.parametrize("conv", ["abs", "norm"])
def test_convergence_tests(orc, conv):
    """EPS_CONV_ABS and EPS_CONV_NORM on a standard problem: every converged pair's true residual ||A x - k x||
    meets tol in the test's own scale (absolute, or relative to ||A||_inf = 12 since ||B|| stays 0 for one matrix),
    and every converged value is an exact eigenvalue.  The stricter absolute test runs longer, so rounding can let
    a second copy of a degenerate eigenvalue converge."""
    m = 10
    csr = matgen.laplacian_3d(m)
    A = matgen.csr_to_dense(*csr)
    kw = dict(hermitian=True, which="LR", nev=6, ncv=24, tol=1e-9, v0=matgen.start_vector(m ** 3, 2))
    rel = orc.solve(*csr, **kw)
    other = orc.solve(*csr, conv=conv, **kw)
    assert rel.reason == 1 and other.reason == 1
    scale = 1.0 if conv == "abs" else 12.0
    for i in range(other.nconv):
        x, lam = other.X[:, i], other.eigr[i]
        assert other.errest[i] < kw["tol"]
        assert np.linalg.norm(A @ x - lam * x) / scale < 10 * kw["tol"]
    ex = matgen.laplacian_eigenvalues([m, m, m])
    for lam in other.eigr[:other.nconv]:  # degenerate copies may appear once rounding splits them
        assert np.min(np.abs(ex - lam)) < 1e-9 * abs(lam)
    assert abs(other.eigr[0] - rel.eigr[0]) < 1e-9 * abs(rel.eigr[0])


def _filtered(vals, g):
    out = [f"{v:.5f}" for v in vals]
    for a, b in g.get("filter", []):
        out = [b if x == a else x for x in out]
    return [float(x) for x in out]


@pytest.mark.parametrize("lock", [True, False])
def test_ex5_markov_golden(orc, lock):
    """ex5.c: the random walk on a triangular grid (m = 15, n = 120), non-Hermitian, largest real, nev 4, with and
    without locking: the digits of ex5_1.out (after the test's own filter)."""
    g = G["ex5_1"]
    csr = matgen.markov_walk(g["m"])
    n = len(csr[0]) - 1
    r = orc.solve(*csr, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"], lock=lock,
                  v0=matgen.start_vector(n, 1))
    assert r.err == 0 and r.reason == 1
    assert _filtered(r.eigr[:4], g) == g["eigenvalues"] and not np.any(r.eigi[:4])


@pytest.mark.parametrize("key,gen", [("test4_1", "lap1d"), ("test6_1", "diag")])
def test_test4_test6_goldens(orc, key, gen):
    """test4.c (1-D Laplacian n = 30) and test6.c (diag(1..30)): HEP, nev 4, largest magnitude."""
    g = G[key]
    n = g["n"]
    csr = matgen.laplacian_1d(n) if gen == "lap1d" else matgen.diagonal(np.arange(1, n + 1, dtype=float))
    r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"], v0=matgen.start_vector(n, 1))
    assert r.err == 0 and r.reason == 1
    assert r5(r.eigr[:4]) == g["eigenvalues"]


def test_oracle_monitor_through_the_c_printer(orc):
    """test23.c TEST 2 on the CPU: the oracle's restart-by-restart values, printed by the library's EPSMonitorFirst,
    are the two lines of test23_2.out after that test's filter."""
    import ctypes
    import re
    import tempfile

    import slepc_gb300 as sg
    sg.build()
    lib = sg.load()
    g = G["test23_2"]
    n = g["n"]
    P, D = ctypes.c_void_p, ctypes.c_double
    rp, ci, va = np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.arange(1, n + 1, dtype=float)
    hist = []
    r = orc.solve(rp, ci, va, hermitian=False, which="LR", nev=1, tol=1e-8, v0=matgen.start_vector(n, 1),
                  monitor=lambda its, nconv, er, ei, es, nest: hist.append((its, nconv, er, ei, es, nest)))
    assert r.reason == 1
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "mon.txt")
        v, vf = P(), P()
        lib.PetscViewerASCIIOpen.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(P)]
        lib.PetscViewerAndFormatCreate.argtypes = [P, ctypes.c_int, ctypes.POINTER(P)]
        lib.EPSMonitorFirst.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(D), ctypes.POINTER(D),
                                        ctypes.POINTER(D), ctypes.c_int, P]
        lib.PetscViewerAndFormatDestroy.argtypes = [ctypes.POINTER(P)]
        lib.PetscViewerDestroy.argtypes = [ctypes.POINTER(P)]
        assert lib.PetscViewerASCIIOpen(0, path.encode(), ctypes.byref(v)) == 0
        assert lib.PetscViewerAndFormatCreate(v, 0, ctypes.byref(vf)) == 0
        eps = sg.EPS().create()
        for its, nconv, er, ei, es, nest in hist:
            assert lib.EPSMonitorFirst(eps.handle, its, nconv, (D * nest)(*er), (D * nest)(*ei), (D * nest)(*es),
                                       nest, vf) == 0
        eps.destroy()
        assert lib.PetscViewerAndFormatDestroy(ctypes.byref(vf)) == 0
        assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0
        lines = open(path).read().splitlines()
    assert [re.sub(r"[0-9]\.[0-9]*e-([0-9]*)", "removed", l) for l in lines] == g["monitor"]


def test_test20_full_basis_golden(orc):
    """test20.c: the smallest eigenvalue of the 1-D Laplacian n = 18 with the default ncv (16) and then with
    ncv = 18 = n (a full basis: the factorisation ends in a breakdown with every eigenvalue converged)."""
    g = G["test20_1"]
    csr = matgen.laplacian_1d(g["n"])
    for ncv, want in zip(g["ncv"], g["eigenvalues"]):
        r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], ncv=ncv, tol=g["tol"],
                      v0=matgen.start_vector(g["n"], 1))
        assert r.err == 0 and r.reason == 1
        assert round(float(r.eigr[0]), 5) == want
    # ncv above n is clamped to n (epssetup.c:337-338)
    r = orc.solve(*csr, hermitian=True, which="SR", nev=2, ncv=40, tol=g["tol"], v0=matgen.start_vector(g["n"], 1))
    assert r.err == 0 and r.reason == 1 and r.ncv == g["n"]


def _npz(name):
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", name))
    return d["rowptr"], d["colidx"], d["vals"]


def test_ex7_general_b_goldens(orc):
    """ex7.c: the GNHEP pencil of the reference's data files bfw62a / bfw62b (B symmetric, not diagonal), B^-1 A with
    a direct solve: the golden eigenvalues within the run's tolerance (tol 1e-8 fixes about 3 decimals of values
    near 2e5) and the dense generalised solve at tol 1e-12; then the pencil (A, A), all eigenvalues 1 in one restart
    as the reference reports."""
    import scipy.linalg as sl
    g = G["ex7_1"]
    A, B = _npz("bfw62a.npz"), _npz("bfw62b.npz")
    v0 = matgen.start_vector(62, 1)
    r = orc.solve(*A, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"], B=B, v0=v0)
    assert r.err == 0 and r.reason == 1
    for (a, b), x, y in zip(g["eigenvalues"], r.eigr, r.eigi):
        assert abs(complex(x, y) - complex(a, b)) <= 10 * g["tol"] * abs(complex(a, b)) + 1e-5
    r = orc.solve(*A, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-12, B=B, v0=v0)
    w = sl.eig(matgen.csr_to_dense(*A), matgen.csr_to_dense(*B), right=False)
    for x, y in zip(r.eigr[:4], r.eigi[:4]):
        z = complex(x, y)
        assert np.min(np.abs(w - z)) <= 1e-10 * abs(z)
    g3 = G["ex7_3"]
    r = orc.solve(*A, hermitian=False, which=g3["which"], nev=g3["nev"], tol=g3["tol"], B=A, v0=v0)
    assert r.err == 0 and r.reason == 1 and r.its == g3["iterations"]
    assert [[round(float(x), 5), round(float(y), 5)] for x, y in zip(r.eigr[:4], r.eigi[:4])] == g3["eigenvalues"]


def test_general_b_ghep(orc):
    """EPS_GHEP with a general SPD B (a tridiagonal mass matrix): against scipy.linalg.eigh(A, B), B-orthonormal
    purified eigenvectors; and a diagonal B through the general path gives the diagonal path's solve exactly."""
    import scipy.linalg as sl
    m = 12
    csr = matgen.laplacian_2d(m, m)
    n = m * m
    rp = [0]
    ci, va = [], []
    for r in range(n):
        for c, v in ((r - 1, 1.0), (r, 4.0), (r + 1, 1.0)):
            if 0 <= c < n:
                ci.append(c)
                va.append(v / 6.0)
        rp.append(len(ci))
    Bc = (np.array(rp, np.int32), np.array(ci, np.int32), np.array(va))
    v0 = matgen.start_vector(n, 3)
    for which in ("LR", "SR"):
        r = orc.solve(*csr, hermitian=True, which=which, nev=5, tol=1e-12, B=Bc, v0=v0)
        assert r.err == 0 and r.reason == 1
        Bd = matgen.csr_to_dense(*Bc)
        w = sl.eigh(matgen.csr_to_dense(*csr), Bd, eigvals_only=True)
        for lam in r.eigr[:5]:
            assert np.min(np.abs(w - lam)) <= 1e-10 * abs(lam)
        X = r.X[:, :r.nconv]
        assert np.abs(X.T @ Bd @ X - np.eye(r.nconv)).max() < 1e-10
    g = G["test1_1"]
    csr = matgen.laplacian_2d(*g["grid"])
    b = matgen.log_mass(324)
    kw = dict(hermitian=True, which="LM", nev=4, tol=g["tol"], conv="norm", v0=matgen.start_vector(324, 1))
    r1 = orc.solve(*csr, bdiag=b, **kw)
    r2 = orc.solve(*csr, B=matgen.diagonal(b), **kw)
    assert r1.its == r2.its and np.array_equal(r1.eigr, r2.eigr)


def test_ghep_harmonic_interior(orc):
    """Interior eigenvalues of a definite pencil: EPS_GHEP with harmonic extraction around a target (the Arnoldi
    variant with the B-inner product, as the reference runs Krylov-Schur with harmonic extraction on a Hermitian
    problem), against scipy.linalg.eigh(A, B): the eigenvalues closest to the target."""
    import scipy.linalg as sl
    m = 14
    csr = matgen.laplacian_2d(m, m)
    n = m * m
    b = 1.0 + matgen.uniform_01(9, n)
    target = 2.05
    r = orc.solve(*csr, hermitian=True, which="TM", nev=4, ncv=40, tol=1e-11, bdiag=b, harmonic=True, target=target,
                  v0=matgen.start_vector(n, 2))
    assert r.err == 0 and r.reason == 1
    w = sl.eigh(matgen.csr_to_dense(*csr), np.diag(b), eigvals_only=True)
    want = w[np.argsort(np.abs(w - target))][:4]
    assert np.allclose(np.sort(r.eigr[:4]), np.sort(want), rtol=1e-9, atol=0)


def test_ex11_deflation_space_golden(orc):
    """ex11.c: the Fiedler vector of a 10 x 10 mesh's graph Laplacian, smallest real, nev 4, restart 0.2, with the
    constant vector (the null space) as deflation space: the eigenvalues ex11_1.out prints, and every computed
    eigenvector orthogonal to the deflation space."""
    g = G["ex11_1"]
    csr = matgen.graph_laplacian_2d(*g["grid"])
    n = len(csr[0]) - 1
    assert np.allclose(np.add.reduceat(csr[2], csr[0][:-1]), 0.0)  # rows sum to zero: the constant is a null vector
    r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=g["tol"],
                     deflation=np.ones(n))
    assert r.reason == 1 and r.nconv >= g["nev"]
    assert [round(v, 5) for v in r.eigr[:g["nev"]]] == g["eigenvalues"]
    assert np.abs(r.X[:, :g["nev"]].sum(axis=0)).max() < 1e-10 * np.sqrt(n)
    # without the deflation space the zero eigenvalue comes first
    r0 = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=g["tol"])
    assert abs(r0.eigr[0]) < 1e-8 and round(r0.eigr[1], 5) == g["eigenvalues"][0]


def test_test24_constrained_laplacian_golden(orc):
    """test24.c: the 1-D Laplacian (n = 30), smallest real, nev 4, EPS_CONV_ABS, with the exact eigenvectors of its
    two lowest eigenvalues as deflation space: the eigenvalues test24_1.out prints (those of the deflated problem,
    2 - 2 cos(k pi / 31) for k = 3..6), every eigenvector orthogonal to the constraints."""
    g = G["test24_1"]
    n, ncon = g["n"], g["ncon"]
    csr = matgen.laplacian_1d(n)
    j = np.arange(1, n + 1)
    C = np.stack([np.sin(np.pi / (n + 1) * j * (i + 1)) * np.sqrt(2.0 / (n + 1)) for i in range(ncon)], axis=1)
    r = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"], conv=g["conv"],
                  v0=matgen.start_vector(n, 1), deflation=C)
    assert r.reason == 1 and r.nconv >= g["nev"]
    assert [round(v, 5) for v in r.eigr[:g["nev"]]] == g["eigenvalues"]
    assert np.abs(C.T @ r.X[:, :g["nev"]]).max() < 1e-10
    exact = [2 - 2 * np.cos(k * np.pi / (n + 1)) for k in range(ncon + 1, ncon + 1 + g["nev"])]
    assert np.allclose(r.eigr[:g["nev"]], exact, rtol=1e-9)
