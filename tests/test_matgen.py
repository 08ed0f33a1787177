"""Synthetic matrix generators: structure, symmetry, closed-form spectra, reproducibility."""
import numpy as np

from slepc_gb300 import matgen


def test_splitmix_reproducible():
    a = matgen.start_vector(1000, 1)
    b = matgen.start_vector(1000, 1)
    assert np.array_equal(a, b)
    assert a.min() >= -1.0 and a.max() < 1.0
    assert not np.array_equal(a, matgen.start_vector(1000, 2))


def test_laplacians_match_closed_form():
    for csr, dims in ((matgen.laplacian_1d(17), [17]), (matgen.laplacian_2d(7, 9), [7, 9]),
                      (matgen.laplacian_3d(5), [5, 5, 5])):
        A = matgen.csr_to_dense(*csr)
        assert np.allclose(A, A.T)
        ev = np.sort(np.linalg.eigvalsh(A))
        assert np.allclose(ev, np.sort(matgen.laplacian_eigenvalues(dims)), atol=1e-12)


def test_config_shapes():
    rp, ci, va = matgen.laplacian_2d(100)
    assert rp.size - 1 == 10000 and ci.size == 49600
    rp, ci, va = matgen.laplacian_3d(16)
    assert ci.size == 7 * 16 ** 3 - 6 * 16 ** 2
    assert np.all(np.diff(rp) > 0)
    for r in range(0, 4096, 97):
        row = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0)


def test_convdiff_closed_form():
    N, Pe = 12, 20.0
    A = matgen.csr_to_dense(*matgen.convection_diffusion_2d(N, Pe))
    ev = np.linalg.eigvals(A)
    assert np.max(np.abs(ev.imag)) < 1e-8
    assert np.allclose(np.sort(ev.real), np.sort(matgen.convdiff_eigenvalues(N, Pe)), atol=1e-8)


def test_chung_lu_symmetric_normalised():
    rp, ci, va = matgen.chung_lu(3000, mean_degree=8, max_degree=500, seed=4, weight_seed=5)
    A = matgen.csr_to_dense(rp, ci, va)
    assert np.allclose(A, A.T)
    assert np.all(np.diag(A) == 0)
    ev = np.linalg.eigvalsh(A)
    assert ev.max() <= 1.0 + 1e-12 and ev.min() >= -1.0 - 1e-12


def test_randdiag():
    rp, ci, va = matgen.laplacian_2d_randdiag(1000, seed=6)
    n = rp.size - 1
    r = int(np.sqrt(1000))
    assert n == r * (-(-1000 // r))
    A = matgen.csr_to_dense(rp, ci, va)
    assert np.allclose(A, A.T)
    assert np.all(np.diag(A) >= 4.0) and np.all(np.diag(A) < 5.0)


def test_chung_lu_native_matches_numpy():
    """The C helper of the Chung-Lu generator reproduces the numpy algorithm bit for bit."""
    for n in (3000, 40000):
        a = matgen.chung_lu(n, native=False)
        b = matgen.chung_lu(n, native=True)
        for x, y in zip(a, b):
            assert x.dtype == y.dtype and np.array_equal(x, y)
