"""GPU: generalised problems A x = k B x with a diagonal B through the C-ABI, and the convergence tests.

The device iterates on C = D^-1/2 A D^-1/2 (EPS_GHEP) or D^-1 A (EPS_GNHEP); the oracle restates the reference's own
formulation (B^-1 A with the B-inner product, start vectors forced into the range of the operator, purified
eigenvectors).  Tolerances: eigenvalues |k - k_ref| <= 1e-10 |k_ref|; B-orthonormality max|X^T B X - I| below
10 tol (test1.c's check); residuals ||A x - k B x|| / (|k| ||x||) <= 10 tol through EPSComputeError."""
import json
import os

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen

pytestmark = pytest.mark.gpu
G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))
PETSC_ERR_SUP, PETSC_ERR_ARG_WRONG = 56, 62


def ghep_eps(csr, b, **kw):
    A = sg.Mat(*csr)
    B = sg.Mat(*matgen.diagonal(b))
    eps = sg.EPS().create()
    eps.setOperators(A, B)
    eps.setProblemType(kw.pop("ptype", sg.EPS.ProblemType.GHEP))
    return eps, A, B


@pytest.mark.parametrize("arith", ["pair", "f64"])
def test_test1_ghep_golden_and_oracle(lib, orc, arith):
    """test1.c on the device: the printed eigenvalues and EPSErrorView(EPS_ERROR_BACKWARD) line of test1_1.out,
    B-orthonormal eigenvectors, and the oracle's eigenvalues and restart count."""
    g = G["test1_1"]
    csr = matgen.laplacian_2d(*g["grid"])
    n = g["grid"][0] * g["grid"][1]
    b = matgen.log_mass(n)
    v0 = matgen.start_vector(n, 1)
    res = sg.solve(csr, B=matgen.diagonal(b), hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"],
                   max_it=g["max_it"], conv="norm", v0=v0, arith=arith)
    eps = res["eps"]
    assert res["reason"] == 1
    assert [round(v, 5) for v in res["eigr"][:4]] == g["eigenvalues"]
    assert eps.errorView(sg.EPS.ErrorType.BACKWARD).splitlines()[:2] == g["errorview"][0]
    X = res["X"]
    assert np.abs(X.T @ (b[:, None] * X) - np.eye(res["nconv"])).max() < 10 * g["tol"]
    ref = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"], max_it=g["max_it"],
                    conv="norm", bdiag=b, v0=v0)
    assert ref.reason == 1 and res["its"] == ref.its
    for i in range(min(res["nconv"], ref.nconv)):
        assert abs(res["eigr"][i] - ref.eigr[i]) <= 1e-10 * abs(ref.eigr[i])
    A = matgen.csr_to_dense(*csr)
    for i in range(res["nconv"]):
        x = X[:, i]
        r = np.linalg.norm(A @ x - res["eigr"][i] * b * x) / (abs(res["eigr"][i]) * np.linalg.norm(x))
        assert r <= 10 * g["tol"]
        assert abs(res["errors"][i] - r) <= 1e-3 * r + 1e-15
        # purified eigenvectors are the oracle's up to the sign of the Ritz vector: x = B^-1 A x / ||B^-1 A x||_B
        xr = ref.X[:, i]
        assert min(np.linalg.norm(x - xr), np.linalg.norm(x + xr)) < 1e-6


def test_ghep_lap3d_random_mass(lib, orc):
    """A 3-D Laplacian 16^3 with B = diag(1 + U[0,1)), largest and smallest ends, against the oracle.  Purification
    (x <- B^-1 A x) amplifies the components along the large eigenvalues by up to k_max / k, so at the smallest end
    the true residuals of the reference's algorithm sit above tol (3.2e-9 at tol 1e-10 here, in the oracle too):
    the device's residuals are held to the oracle's."""
    m = 16
    n = m ** 3
    csr = matgen.laplacian_3d(m)
    b = 1.0 + matgen.uniform_01(5, n)
    v0 = matgen.start_vector(n, 4)
    A = matgen.csr_to_dense(*csr)
    for which in ("LR", "SR"):
        res = sg.solve(csr, B=matgen.diagonal(b), hermitian=True, which=which, nev=8, ncv=32, tol=1e-10, v0=v0)
        ref = orc.solve(*csr, hermitian=True, which=which, nev=8, ncv=32, tol=1e-10, bdiag=b, v0=v0)
        assert res["reason"] == 1 and ref.reason == 1
        for i in range(8):
            assert abs(res["eigr"][i] - ref.eigr[i]) <= 1e-10 * abs(ref.eigr[i]), (which, i)
        X = res["X"]
        assert np.abs(X.T @ (b[:, None] * X) - np.eye(res["nconv"])).max() < 1e-9
        ref_err = max(np.linalg.norm(A @ ref.X[:, i] - ref.eigr[i] * b * ref.X[:, i])
                      / (abs(ref.eigr[i]) * np.linalg.norm(ref.X[:, i])) for i in range(8))
        assert max(res["errors"][:8]) <= 2.0 * ref_err + 1e-10, (which, max(res["errors"][:8]), ref_err)


def test_gnhep_convdiff(lib, orc):
    """EPS_GNHEP (the default with two matrices) on the convection-diffusion operator with a random diagonal B."""
    N = 40
    n = N * N
    csr = matgen.convection_diffusion_2d(N, 2.0)
    b = 1.0 + matgen.uniform_01(11, n)
    v0 = matgen.start_vector(n, 2)
    A = sg.Mat(*csr)
    B = sg.Mat(*matgen.diagonal(b))
    eps = sg.EPS().create()
    eps.setOperators(A, B)  # no problem type: EPS_GNHEP
    eps.setDimensions(6)
    eps.setTolerances(1e-11)
    eps.setWhichEigenpairs("LR")
    eps.setInitialSpace(v0)
    eps.solve()
    assert eps.getConvergedReason() == 1
    ref = orc.solve(*csr, hermitian=False, which="LR", nev=6, tol=1e-11, bdiag=b, v0=v0)
    assert ref.reason == 1
    for i in range(6):
        z = complex(eps.getEigenvalue(i))
        assert abs(z - complex(ref.eigr[i], ref.eigi[i])) <= 1e-10 * abs(z)
        assert eps.computeError(i) <= 1e-9


@pytest.mark.parametrize("conv", ["abs", "norm"])
def test_convergence_tests_match_oracle(lib, orc, conv):
    """EPS_CONV_ABS / EPS_CONV_NORM on a standard problem with a simple spectrum (3-D Laplacian 16^3 plus a random
    diagonal): the device's restart count and eigenvalues follow the oracle's."""
    m = 16
    csr = matgen.laplacian_3d_randdiag(m, 3)
    v0 = matgen.start_vector(m ** 3, 2)
    kw = dict(hermitian=True, which="LR", nev=6, ncv=24, tol=1e-9, v0=v0)
    res = sg.solve(csr, conv=conv, **kw)
    ref = orc.solve(*csr, conv=conv, **kw)
    assert res["reason"] == 1 and ref.reason == 1
    assert res["eps"].getConvergenceTest() == {"abs": 0, "norm": 2}[conv]
    assert res["its"] == ref.its
    for i in range(min(res["nconv"], ref.nconv)):
        assert abs(res["eigr"][i] - ref.eigr[i]) <= 1e-9 * abs(ref.eigr[i])


def test_generalised_errors(lib):
    """A non-diagonal B that is not positive definite for EPS_GHEP, a non-diagonal B above the dense size limit, an
    indefinite diagonal B for EPS_GHEP, and the batched engine with B: errors, not solves."""
    csr = matgen.laplacian_1d(50)
    eps, A, B = ghep_eps(csr, np.ones(50))
    eps.setDimensions(2)
    eps.destroy()
    rp, ci, va = matgen.laplacian_1d(50)
    nondiag = sg.Mat(rp, ci, -va)  # negative definite
    eps = sg.EPS().create()
    eps.setOperators(sg.Mat(*csr), nondiag)
    eps.setProblemType(sg.EPS.ProblemType.GHEP)
    with pytest.raises(sg.SlepcError) as e:
        eps.setUp()
    assert e.value.code == PETSC_ERR_ARG_WRONG
    big = matgen.laplacian_1d(3000)
    eps = sg.EPS().create()
    eps.setOperators(sg.Mat(*big), sg.Mat(*big))
    eps.setProblemType(sg.EPS.ProblemType.GNHEP)
    with pytest.raises(sg.SlepcError) as e:
        eps.setUp()
    assert e.value.code == PETSC_ERR_SUP
    b = np.ones(50)
    b[7] = -1.0
    eps, A, B = ghep_eps(csr, b)
    with pytest.raises(sg.SlepcError) as e:
        eps.setUp()
    assert e.value.code == PETSC_ERR_ARG_WRONG
    eps, A, B = ghep_eps(csr, np.ones(50))
    eps.setDimensions(2)
    eps.setUp()
    with pytest.raises(sg.SlepcError) as e:
        sg.solve_batch([eps])
    assert e.value.code == PETSC_ERR_SUP


def _npz(name):
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", name))
    return d["rowptr"], d["colidx"], d["vals"]


@pytest.mark.parametrize("arith", ["f64", "pair"])
def test_ex7_general_b_on_gpu(lib, orc, arith):
    """ex7.c: the GNHEP pencil bfw62a / bfw62b (B symmetric indefinite, not diagonal): C = B^-1 A formed on the
    device (LU with partial pivoting, then the 62 solves). The golden eigenvalues within the run's tolerance, the
    oracle's per-step direct solve and scipy's dense generalised solve at tol 1e-12, EPSComputeError's residual
    ||A x - k B x|| with the user's B; then the pencil (A, A): every eigenvalue 1 (ex7_3.out prints one restart; here
    C = A^-1 A is the identity up to rounding, and the Krylov space grows out of that rounding, so the restart count
    follows the arithmetic's rounding: one to three were seen). A singular B is an error at set-up."""
    import scipy.linalg as sl
    g = G["ex7_1"]
    A, B = _npz("bfw62a.npz"), _npz("bfw62b.npz")
    v0 = matgen.start_vector(62, 1)
    res = sg.solve(A, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"], B=B, v0=v0, arith=arith)
    assert res["reason"] == 1 and res["nconv"] >= g["nev"]
    got = res["eigr"] + 1j * res["eigi"]
    for a, b in g["eigenvalues"]:
        z = complex(a, b)
        assert np.min(np.abs(got - z)) <= 10 * g["tol"] * abs(z) + 1e-5, z
    tight = sg.solve(A, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-12, B=B, v0=v0, arith=arith)
    w = sl.eig(matgen.csr_to_dense(*A), matgen.csr_to_dense(*B), right=False)
    ref = orc.solve(*A, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-12, B=B, v0=v0)
    refz = np.asarray(ref.eigr[:ref.nconv]) + 1j * np.asarray(ref.eigi[:ref.nconv])
    for x, y in zip(tight["eigr"][:4], tight["eigi"][:4]):
        z = complex(x, y)
        assert np.min(np.abs(w - z)) <= 1e-10 * abs(z)
        assert np.min(np.abs(refz - z)) <= 1e-10 * abs(z)
    assert max(tight["errors"][:4]) <= 1e-10
    g3 = G["ex7_3"]
    r3 = sg.solve(A, hermitian=False, which=g3["which"], nev=g3["nev"], tol=g3["tol"], B=A, v0=v0, arith=arith)
    assert r3["reason"] == 1 and r3["its"] <= g3["iterations"] + 4
    assert [[round(float(x), 5), round(float(y), 5)] for x, y in zip(r3["eigr"][:4], r3["eigi"][:4])] == \
        g3["eigenvalues"]
    rp, ci, va = B
    sing = (rp, ci, va.copy())
    sing[2][rp[5]:rp[6]] = 0.0  # a zero row: B singular
    with pytest.raises(sg.SlepcError) as e:
        sg.solve(A, hermitian=False, which="LM", nev=2, B=sing, v0=v0)
    assert e.value.code == PETSC_ERR_ARG_WRONG


def test_ghep_general_b_on_gpu(lib, orc):
    """EPS_GHEP with a non-diagonal SPD B (a tridiagonal mass matrix): B = L L^T on the device and C = L^-1 A L^-T,
    against scipy.linalg.eigh(A, B) and the oracle's B-inner-product Lanczos, B-orthonormal purified eigenvectors
    (both ends of the spectrum), EPSComputeError with the user's B, and the device eigenvector array."""
    import scipy.linalg as sl
    m = 12
    csr = matgen.laplacian_2d(m, m)
    n = m * m
    rp, ci, va = [0], [], []
    for r in range(n):
        for c, v in ((r - 1, 1.0), (r, 4.0), (r + 1, 1.0)):
            if 0 <= c < n:
                ci.append(c)
                va.append(v / 6.0)
        rp.append(len(ci))
    Bc = (np.array(rp, np.int32), np.array(ci, np.int32), np.array(va))
    Bd = matgen.csr_to_dense(*Bc)
    w = sl.eigh(matgen.csr_to_dense(*csr), Bd, eigvals_only=True)
    v0 = matgen.start_vector(n, 3)
    for which, arith in (("LR", "f64"), ("SR", "f64"), ("LR", "pair")):
        res = sg.solve(csr, hermitian=True, which=which, nev=5, tol=1e-12, B=Bc, v0=v0, arith=arith)
        assert res["reason"] == 1 and res["nconv"] >= 5
        for lam in res["eigr"][:5]:
            assert np.min(np.abs(w - lam)) <= 1e-10 * abs(lam)
        ref = orc.solve(*csr, hermitian=True, which=which, nev=5, tol=1e-12, B=Bc, v0=v0)
        for lam in ref.eigr[:5]:
            assert np.min(np.abs(res["eigr"][:res["nconv"]] - lam)) <= 1e-10 * abs(lam)
        X = res["X"][:, :res["nconv"]]
        assert np.abs(X.T @ Bd @ X - np.eye(res["nconv"])).max() < 1e-10
        assert max(res["errors"][:5]) <= 1e-10
        Xd = res["eps"].copyDeviceEigenvectors()
        assert np.allclose(Xd[:, :res["nconv"]], X, rtol=0, atol=1e-13)
