"""GPU: EPSGB300SolveBatch, the batched engine (many problems per launch, one restart cycle per CUDA graph).

Every instance runs the single-problem path's device bodies with the same block partition, so a problem's results
are bit-identical alone (EPSSolve with the FP64 QR projected solver, or a batch of one) and inside any mix; the
eigenvalues are also checked against the oracle at 1e-10 and the residuals against tol."""
import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen, verify

pytestmark = pytest.mark.gpu


def make(csr, hermitian, which, nev, ncv, tol, seed, ds=None, restart=None):
    A = sg.Mat(*csr)
    eps = sg.EPS().create()
    eps.setOperators(A)
    eps.setProblemType(sg.EPS.ProblemType.HEP if hermitian else sg.EPS.ProblemType.NHEP)
    eps.setDimensions(nev, ncv)
    eps.setTolerances(tol)
    eps.setWhichEigenpairs(which)
    if ds:
        eps.setProjectedSolver(ds)
    if restart:
        eps.setRestartMethod(restart)
    eps.setInitialSpace(matgen.start_vector(len(csr[0]) - 1, seed))
    eps._A = A  # keep the matrix alive as long as the solver
    return eps


def results(eps):
    nconv = eps.getConverged()
    n = eps._A.m
    vals, vecs = [], []
    for i in range(nconv):
        x = np.zeros(n)
        v = eps.getEigenpair(i, x)
        vals.append(v)
        vecs.append(x)
    return nconv, eps.getIterationNumber(), eps.getConvergedReason(), vals, vecs


def mixed_problems():
    probs = []
    for i, n in enumerate([1000, 1500, 2304, 3000, 4096]):
        probs.append((matgen.laplacian_2d_randdiag(n, 100 + i), True, "LM", 8, 24, 1e-10, 6 + i))
    # Pe = 2 keeps the non-symmetric eigenvalues well conditioned (the similarity to a symmetric operator grows like
    # (1 + Pe h)^N): two summation orders then agree to the parity tolerance, not to cond * tol
    probs.append((matgen.convection_diffusion_2d(40, 2.0), False, "LR", 6, 24, 1e-10, 3))
    probs.append((matgen.laplacian_3d(14), True, "SR", 6, 24, 1e-10, 9))
    return probs


def test_batch_equals_single_problem_path(lib):
    """With one tile per virtual block the batch partitions every reduction exactly as the single-problem kernels
    do, so the results are bit-identical to EPSSolve with the same (QR) projected solver and the same (CUDA-core)
    restart kernel."""
    saved = sg.batch_get_tuning()
    try:
        sg.batch_set_tuning([1] * sg.BATCH_BUCKETS)
        probs = mixed_problems()
        batch = [make(*p) for p in probs]
        sg.solve_batch(batch)
        for p, b in zip(probs, batch):
            alone = make(*p, ds="qr", restart="pair")
            alone.solve()
            ra, rb = results(alone), results(b)
            assert ra[0] == rb[0] and ra[1] == rb[1] and ra[2] == rb[2] == 1
            assert ra[3] == rb[3], (ra[3], rb[3])
            for xa, xb in zip(ra[4], rb[4]):
                assert np.array_equal(xa, xb)
    finally:
        sg.batch_set_tuning(saved)


def test_batch_tuned_matches_single_problem_path(lib):
    """With the default tuning (several tiles per virtual block) only the summation order changes; both runs
    converge to tol 1e-10, and their eigenvalues agree within the parity tolerance 1e-10 (relative)."""
    probs = mixed_problems()
    batch = [make(*p) for p in probs]
    sg.solve_batch(batch)
    for p, b in zip(probs, batch):
        nev = p[3]
        alone = make(*p, ds="qr")
        alone.solve()
        ra, rb = results(alone), results(b)
        assert ra[2] == rb[2] == 1 and min(ra[0], rb[0]) >= nev
        # set-based: degenerate spectra (the 3-D Laplacian) may gain copies in a different order
        vb = np.asarray(rb[3])
        for va in ra[3][:nev]:
            assert np.min(np.abs(vb - va)) <= 1e-10 * abs(va)


def test_batch_alone_equals_in_mix(lib):
    probs = mixed_problems()
    mix = [make(*p) for p in probs]
    sg.solve_batch(mix)
    for k in (0, 3, 5):
        one = [make(*probs[k])]
        sg.solve_batch(one)
        r1, rm = results(one[0]), results(mix[k])
        assert r1[:3] == rm[:3] and r1[3] == rm[3]
        for xa, xb in zip(r1[4], rm[4]):
            assert np.array_equal(xa, xb)


def test_batch_parity_with_oracle(lib, orc):
    probs = mixed_problems()
    batch = [make(*p) for p in probs]
    sg.solve_batch(batch)
    for (csr, herm, which, nev, ncv, tol, seed), b in zip(probs, batch):
        nconv, its, reason, vals, vecs = results(b)
        assert reason == 1 and nconv >= nev
        ref = orc.solve(*csr, hermitian=herm, which=which, nev=nev, ncv=ncv, tol=tol,
                        v0=matgen.start_vector(len(csr[0]) - 1, seed))
        refv = np.asarray(ref.eigr[:ref.nconv]) + 1j * np.asarray(ref.eigi[:ref.nconv])
        for v in vals[:nev]:
            assert np.min(np.abs(refv - v)) / abs(v) <= 1e-10
        real = [(v, x) for v, x in zip(vals, vecs) if not isinstance(v, complex)]
        if real:  # host check: scipy.sparse on the CSR arrays
            r_a, _ = verify.residuals(csr, [v for v, _ in real], np.stack([x for _, x in real], axis=1))
            assert r_a.max() <= tol


def test_batch_zero_start_vector_error(lib):
    csr = matgen.laplacian_1d(200)
    eps = make(csr, True, "LM", 2, 10, 1e-8, 1)
    eps.setInitialSpace(np.zeros(200))
    with pytest.raises(sg.SlepcError) as ei:
        sg.solve_batch([eps])
    assert ei.value.code == 77


def test_batch_precision_form(lib):
    """The FP32-storage variant in the batch: FP32 phase, FP64 recheck, refinement sweep through the engine again;
    mixed with pair-arithmetic problems in the same batch.  Eigenvalues against dense FP64 solves."""
    probs = [(matgen.laplacian_2d_randdiag(n, 300 + n % 97), True, "LM", 8, 24, 1e-10, 40 + k)
             for k, n in enumerate([1500, 2600, 3600])]
    eps = [make(*p) for p in probs]
    for e in eps[:2]:
        e.setArithmetic("f32")
    sg.solve_batch(eps)
    for p, e in zip(probs, eps):
        nconv, its, reason, vals, vecs = results(e)
        assert reason == 1 and nconv >= p[3]
        dense = np.linalg.eigvalsh(matgen.csr_to_dense(*p[0]))
        for v in vals[:p[3]]:
            assert np.min(np.abs(dense - v)) / abs(v) <= 1e-10
        r_a, _ = verify.residuals(p[0], list(vals), np.stack(vecs, axis=1))  # host, scipy.sparse
        assert r_a.max() <= 1e-10
    for e in eps[:2]:
        st = e.getStats()
        assert 0 < st["precision_steps"] < st["krylov_steps"]
    assert eps[2].getStats()["precision_steps"] == 0


def test_wide_batch_equals_single_problem_path(lib):
    """An engine wider than 80 columns (ncv 100: the dot kernel's 144-column tiling) stays bit-identical to EPSSolve
    with the same projected solver and restart kernel, for symmetric and non-symmetric instances."""
    saved = sg.batch_get_tuning()
    try:
        sg.batch_set_tuning([1] * sg.BATCH_BUCKETS)
        probs = [(matgen.laplacian_2d_randdiag(n, 200 + i), True, "LR", 40, 100, 1e-10, 20 + i)
                 for i, n in enumerate([3000, 5000, 8000])]
        probs.append((matgen.convection_diffusion_2d(60, 2.0), False, "LR", 30, 100, 1e-10, 5))
        probs.append((matgen.laplacian_2d_randdiag(2000, 7), True, "LM", 8, 24, 1e-10, 8))  # a narrow one beside
        batch = [make(*p) for p in probs]
        sg.solve_batch(batch)
        for p, b in zip(probs, batch):
            alone = make(*p, ds="qr", restart="pair")
            alone.solve()
            ra, rb = results(alone), results(b)
            assert ra[0] == rb[0] and ra[1] == rb[1] and ra[2] == rb[2] == 1
            assert ra[3] == rb[3], (ra[3], rb[3])
            for xa, xb in zip(ra[4], rb[4]):
                assert np.array_equal(xa, xb)
    finally:
        sg.batch_set_tuning(saved)
