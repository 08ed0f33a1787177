"""GPU: the skewed symmetric workload (Chung-Lu normalised adjacency, power-law degrees).

Rows above 4096 nonzeros go through the segmented SpMV (one warp per 2048-nonzero segment, in-order merge); the
solve must match the oracle's eigenvalues (set-based, relative 1e-10: lambda = 1 has one copy per connected
component, and single-vector Krylov finds copies only through rounding), with residuals within tol and an
orthonormal basis, in both arithmetics."""
import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen, verify

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("arith", ["pair", "f64"])
def test_chung_lu_parity(lib, orc, arith):
    n = 60000
    csr = matgen.chung_lu(n)
    assert (np.diff(csr[0]) > 4096).sum() > 0  # the segmented path is exercised
    v0 = matgen.start_vector(n, 4)
    res = sg.solve(csr, hermitian=True, which="LR", nev=16, ncv=48, tol=1e-10, v0=v0, arith=arith)
    ref = orc.solve(*csr, hermitian=True, which="LR", nev=16, ncv=48, tol=1e-10, v0=v0)
    assert res["reason"] == 1 and res["nconv"] >= 16
    refv = np.asarray(ref.eigr[:ref.nconv])
    for v in res["eigr"][:16]:
        assert np.min(np.abs(refv - v)) / abs(v) <= 1e-10
    for v in refv[:16]:
        assert np.min(np.abs(res["eigr"] - v)) / abs(v) <= 1e-10
    assert abs(res["eigr"][0] - 1.0) <= 1e-12
    r_a, _ = verify.residuals(csr, res["eigr"][:res["nconv"]], res["X"][:, :res["nconv"]])  # host, scipy.sparse
    assert r_a.max() <= 1e-10
    assert verify.orthogonality(res["X"][:, :res["nconv"]]) <= 1e-12
