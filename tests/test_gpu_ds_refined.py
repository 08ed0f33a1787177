"""GPU: the mixed-precision symmetric projected solver (FP32 QL + FP64 Ogita-Aishima refinement) against the FP64
QL solver of the reference's algorithm, on spectra with well-separated, closely spaced and nearly degenerate
eigenvalues, with and without locking.

Both runs start from the same vector; they may take different restart paths once rounding differs, so the check is
on results: the same converged eigenvalues (relative 1e-10, set-based), residuals ||Ax - lam x|| / (||A|| |lam|)
<= tol, ||V^T V - I||_max <= 1e-12."""
import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen, verify

pytestmark = pytest.mark.gpu


def residuals_ok(csr, res, tol):
    """Host check: ||A x - lam x|| / (||A||_inf |lam|) with scipy.sparse on the CSR arrays."""
    m = res["nconv"]
    r_a, _ = verify.residuals(csr, res["eigr"][:m], res["X"][:, :m])
    return bool(r_a.max() <= tol)


def set_close(a, b, tol):
    b = np.asarray(b)
    return max(np.min(np.abs(b - v)) / abs(v) for v in a) <= tol


def wilkinson_plus(m):
    """W_{2m+1}^+: diagonal |i - m|, unit off-diagonals; its largest eigenvalues come in nearly equal pairs."""
    n = 2 * m + 1
    rows, cols, vals = [], [], []
    for i in range(n):
        if i > 0:
            rows.append(i); cols.append(i - 1); vals.append(1.0)
        rows.append(i); cols.append(i); vals.append(float(abs(i - m)))
        if i < n - 1:
            rows.append(i); cols.append(i + 1); vals.append(1.0)
    rp = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rp, np.asarray(rows) + 1, 1)
    return np.cumsum(rp).astype(np.int32), np.asarray(cols, dtype=np.int32), np.asarray(vals)


CASES = {
    "lap2d_60_LR": (lambda: matgen.laplacian_2d(60), dict(which="LR", nev=16, ncv=48, tol=1e-10)),
    "lap3d_20_SR": (lambda: matgen.laplacian_3d(20), dict(which="SR", nev=12, ncv=40, tol=1e-10)),
    "lap3d_24_LR_nolock": (lambda: matgen.laplacian_3d(24), dict(which="LR", nev=20, ncv=64, tol=1e-10,
                                                                lock=False)),
    "randdiag_LM": (lambda: matgen.laplacian_2d_randdiag(2500, 7), dict(which="LM", nev=10, ncv=32, tol=1e-10)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_refined_matches_qr(lib, name):
    gen, kw = CASES[name]
    csr = gen()
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 11)
    a = sg.solve(csr, hermitian=True, v0=v0, ds="refined", **kw)
    b = sg.solve(csr, hermitian=True, v0=v0, ds="qr", **kw)
    nev = kw["nev"]
    for r in (a, b):
        assert r["reason"] == 1 and r["nconv"] >= nev
        assert residuals_ok(csr, r, kw["tol"])
        assert verify.orthogonality(r["X"][:, :r["nconv"]]) <= 1e-12
    assert set_close(a["eigr"][:nev], b["eigr"], 1e-10)
    assert set_close(b["eigr"][:nev], a["eigr"], 1e-10)
    # the same number of restarts, give or take a few, when the paths agree
    assert abs(a["its"] - b["its"]) <= max(2, b["its"] // 5)


@pytest.mark.parametrize("lock", [True, False])
def test_refined_nearly_degenerate_pairs(lib, lock):
    csr = wilkinson_plus(200)
    n = len(csr[0]) - 1
    dense = np.linalg.eigvalsh(matgen.csr_to_dense(*csr))
    res = sg.solve(csr, hermitian=True, which="LR", nev=8, ncv=40, tol=1e-12, v0=matgen.start_vector(n, 4),
                   ds="refined", lock=lock)
    assert res["reason"] == 1 and res["nconv"] >= 8
    assert set_close(res["eigr"][:8], dense, 1e-12)
    assert residuals_ok(csr, res, 1e-12)
    assert verify.orthogonality(res["X"][:, :res["nconv"]]) <= 1e-12


@pytest.mark.parametrize("arith,ds", [("f64", "qr"), ("pair", "qr"), ("f64", "refined"), ("f64", "auto"),
                                     ("pair", "auto")])
def test_lap3d64_nev50_ncv128_host_parity(lib, arith, ds):
    """The 128^3 workload's shape at 64^3 (nev 50, ncv 128, tol 1e-10, largest algebraic): a degenerate spectrum
    with pairs just outside the cluster threshold of the mixed-precision projected solver, where its refinement
    alone left mixed Ritz vectors (now caught by its check and redone in FP64).  Checked on the host: eigenvalues
    against the closed form (set-based over distinct values), residuals with scipy.sparse, ||X^T X - I|| in
    numpy."""
    m = 64
    csr = matgen.laplacian_3d(m)
    res = sg.solve(csr, hermitian=True, which="LR", nev=50, ncv=128, tol=1e-10, v0=matgen.start_vector(m ** 3, 2),
                   arith=arith, ds=ds)
    assert res["reason"] == 1 and res["nconv"] >= 50
    k = res["nconv"]
    p = verify.parity_block(csr, res["eigr"][:k], res["X"][:, :k], matgen.laplacian_eigenvalues([m] * 3), "LR", 50,
                            1e-10)
    assert p["ok"], p
    _, r_l = verify.residuals(csr, res["eigr"][:k], res["X"][:, :k])
    assert r_l.max() <= 2e-10, r_l.max()  # ||Ax - lam x|| / |lam|: the convergence test's own measure, at tol


def test_auto_projected_solver_is_the_default_and_matches_qr(lib):
    """The default projected solver (auto) on the 100^2 Laplacian of the small workload, beside the FP64 QR solver:
    both pass the parity block against the closed form (the spectrum has multiplicity 2, so which copies converge
    first differs with rounding; the distinct wanted values are found by both), host residuals at tol."""
    csr = matgen.laplacian_2d(100)
    v0 = matgen.start_vector(10000, 1)
    exact = matgen.laplacian_eigenvalues([100, 100])
    for ds in (None, "qr"):
        r = sg.solve(csr, hermitian=True, which="LM", nev=10, ncv=32, tol=1e-10, v0=v0, arith="f64", ds=ds)
        assert r["reason"] == 1 and r["nconv"] >= 10
        k = r["nconv"]
        p = verify.parity_block(csr, r["eigr"][:k], r["X"][:, :k], exact, "LM", 10, 1e-10)
        assert p["ok"], (ds, p)
        if ds == "qr":
            assert r["stats"]["ds_fallbacks"] == 0
