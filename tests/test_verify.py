"""CPU: the host-side parity checks (slepc_gb300.verify) on dense LAPACK results of small problems, and the checks
catching a planted error."""
import numpy as np
import scipy.linalg as sl

from slepc_gb300 import matgen, verify


def _dense_pairs(csr, which, nev):
    A = matgen.csr_to_dense(*csr)
    w, X = sl.eigh(A)
    order = np.argsort(-w) if which == "LR" else np.argsort(w)
    return w[order[:nev]], X[:, order[:nev]]


def test_parity_block_on_exact_pairs():
    csr = matgen.laplacian_2d(12, 9)
    lams, X = _dense_pairs(csr, "LR", 6)
    exact = matgen.laplacian_eigenvalues([12, 9])
    p = verify.parity_block(csr, lams, X, exact, "LR", 6, 1e-10)
    assert p["ok"], p
    assert p["max_rel_eig_err"] < 1e-13 and p["max_rel_residual"] < 1e-13 and p["orth_err"] < 1e-13
    assert p["distinct_found"] == p["distinct_wanted"] >= 1


def test_degenerate_spectrum_matches_by_distinct_values():
    # the square grid has multiplicity 2: one copy per distinct eigenvalue is enough
    csr = matgen.laplacian_2d(10)
    exact = matgen.laplacian_eigenvalues([10, 10])
    dv = verify.distinct(np.sort(exact)[::-1])
    m = verify.match_spectrum(dv[:5], exact, "LR", 6)
    assert m["ok"], m
    # a missing distinct eigenvalue is caught
    m2 = verify.match_spectrum([dv[0], dv[2], dv[3], dv[4]], exact, "LR", 6)
    assert not m2["ok"] and m2["distinct_found"] < m2["distinct_wanted"]


def test_planted_errors_are_caught():
    csr = matgen.laplacian_1d(40)
    lams, X = _dense_pairs(csr, "LR", 4)
    exact = matgen.laplacian_eigenvalues([40])
    bad = lams.copy()
    bad[1] *= 1 + 1e-8
    assert not verify.parity_block(csr, bad, X, exact, "LR", 4, 1e-10)["ok"]
    Xb = X.copy()
    Xb[:, 2] += 1e-9 * X[:, 0]
    p = verify.parity_block(csr, lams, Xb, exact, "LR", 4, 1e-10)
    assert not p["ok"] and p["orth_err"] > 1e-12


def test_convdiff_closed_form_against_dense():
    N, pe = 9, 10.0
    csr = matgen.convection_diffusion_2d(N, pe)
    w = np.linalg.eigvals(matgen.csr_to_dense(*csr))
    assert np.max(np.abs(w.imag)) < 1e-8
    exact = matgen.convdiff_eigenvalues(N, pe)
    m = verify.match_spectrum(np.sort(w.real)[::-1][:5], exact, "LR", 5, rel_tol=1e-9)
    assert m["ok"], m
