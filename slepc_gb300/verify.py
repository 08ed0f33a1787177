"""Host-side checks of a solve's results that do not run through the device path.

Everything here is numpy/scipy on the host: the eigenvectors come back through EPSGetEigenpair, the operator is the
caller's own CSR arrays, and the exact spectra are closed forms.  The device's own MatMult and Gram-Schmidt kernels
are never used, so these checks are independent of the code they check.

  match_spectrum   set-based eigenvalue parity against an exact spectrum (degenerate spectra give one Krylov copy
                   per distinct eigenvalue, so matching is by distinct values, with the converged count reported)
  residuals        ||A x - lam x|| / (||A||_inf |lam|) and ||A x - lam x|| / |lam| with scipy.sparse
  orthogonality    ||X^T X - I||_max of the returned eigenvectors (Hermitian problems)

The residual follows EPSComputeResidualNorm_Private (src/eps/interface/epssolve.c:666-718, real case) and the
relative error of EPSComputeError (epssolve.c:742-815); the orthogonality measure is the one of
BVOrthogonalize's tests (src/sys/classes/bv/tests/test2.c: ||V^T V - I||).
"""
from __future__ import annotations

import numpy as np


def _order(vals, which):
    vals = np.asarray(vals, dtype=float)
    if which in ("LR", "LA"):
        return np.sort(vals)[::-1]
    if which in ("SR", "SA"):
        return np.sort(vals)
    if which == "LM":
        return vals[np.argsort(-np.abs(vals), kind="stable")]
    if which == "SM":
        return vals[np.argsort(np.abs(vals), kind="stable")]
    raise ValueError(f"unsupported criterion {which}")


def distinct(vals, rel=1e-9):
    """Distinct values of a sorted-by-criterion list: a value within rel of one already kept is a copy."""
    out = []
    for v in vals:
        if not any(abs(v - u) <= rel * max(abs(u), 1e-300) for u in out):
            out.append(float(v))
    return out


def match_spectrum(computed, exact, which, nev, rel_tol=1e-10):
    """Set-based parity of computed (real) eigenvalues against the exact spectrum.

    Returns a dict: max_rel_eig_err (every computed value against its nearest exact eigenvalue), the distinct
    wanted eigenvalues (the first ones by `which` until nev copies are covered), how many of them were found, and
    ok = every computed value within rel_tol and every distinct wanted value found within rel_tol."""
    computed = np.asarray(computed, dtype=float)
    ex = _order(exact, which)
    errs = [float(np.min(np.abs(ex - lam)) / abs(lam)) for lam in computed]
    max_err = max(errs) if errs else float("inf")
    # the wanted distinct values: walk the exact spectrum in criterion order until nev values (with multiplicity)
    # are covered; each must appear among the computed values
    wanted, covered = [], 0
    dv = distinct(ex[: max(4 * nev, nev + 64)])
    for v in dv:
        if covered >= nev:
            break
        wanted.append(v)
        covered += int(np.sum(np.abs(ex - v) <= 1e-9 * abs(v)))
    found = sum(1 for v in wanted if computed.size and np.min(np.abs(computed - v)) / abs(v) <= rel_tol)
    return {"max_rel_eig_err": max_err, "distinct_wanted": len(wanted), "distinct_found": found,
            "converged": int(computed.size), "ok": bool(max_err <= rel_tol and found == len(wanted))}


def norm_inf(csr):
    rp, ci, va = csr
    if va.size == 0:
        return 0.0
    return float(np.max(np.add.reduceat(np.abs(va), rp[:-1])))


def csr_matrix(csr, n=None):
    import scipy.sparse as sp

    rp, ci, va = csr
    m = len(rp) - 1
    return sp.csr_matrix((va, ci, rp), shape=(m, n if n else m))


def residuals(csr, lams, X, chunk=16):
    """Per eigenpair (real): ||A x - lam x||_2 / (||A||_inf |lam|) and ||A x - lam x||_2 / |lam| (x as returned,
    unit norm).  Columns are processed in chunks to bound host memory."""
    A = csr_matrix(csr)
    nrm = norm_inf(csr)
    lams = np.asarray(lams, dtype=float)
    r_a, r_l = [], []
    for c0 in range(0, X.shape[1], chunk):
        Xc = X[:, c0:c0 + chunk]
        R = A @ Xc - Xc * lams[c0:c0 + chunk]
        rn = np.linalg.norm(R, axis=0)
        for i, r in enumerate(rn):
            lam = abs(lams[c0 + i])
            r_a.append(float(r / (nrm * lam)))
            r_l.append(float(r / lam))
    return np.array(r_a), np.array(r_l)


def orthogonality(X):
    """||X^T X - I||_max."""
    if X.shape[1] == 0:
        return 0.0
    G = X.T @ X
    return float(np.max(np.abs(G - np.eye(X.shape[1]))))


def parity_block(csr, lams, X, exact, which, nev, tol, hermitian=True, checked="closed form"):
    """The bench's parity object: eigenvalues against the exact spectrum, residuals and orthogonality on the
    host."""
    m = match_spectrum(lams, exact, which, nev)
    r_a, r_l = residuals(csr, lams, X)
    out = {"checked": checked, "max_rel_eig_err": m["max_rel_eig_err"], "distinct_wanted": m["distinct_wanted"],
           "distinct_found": m["distinct_found"], "converged": m["converged"],
           "max_rel_residual": float(r_a.max()) if r_a.size else None,
           "max_residual_over_lambda": float(r_l.max()) if r_l.size else None,
           "orth_err": orthogonality(X) if hermitian else None, "tol": tol}
    out["ok"] = bool(m["ok"] and (out["max_rel_residual"] is None or out["max_rel_residual"] <= tol)
                     and (out["orth_err"] is None or out["orth_err"] <= 1e-12))
    return out
