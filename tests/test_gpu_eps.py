"""GPU parity: EPSSolve through the C-ABI against the oracle, the reference's goldens and closed-form spectra.

Tolerances: eigenvalues |lam - lam_ref| / |lam_ref| <= 1e-10 (set-based: degenerate spectra give one copy per
distinct eigenvalue, as the reference's ex2_1.out shows), relative residual ||Ax - lam x|| / (||A|| |lam|) <= tol,
||V^T V - I||_max <= 1e-12."""
import json
import re
import os

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen, verify

pytestmark = pytest.mark.gpu
G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))


def run(csr, **kw):
    return sg.solve(csr, **kw)


def rel_match(vals, ref, tol):
    ref = np.asarray(ref)
    return max(np.min(np.abs(ref - v)) / abs(v) for v in vals) <= tol


def check_residuals(csr, res, tol):
    """||A x - lam x|| / (||A||_inf |lam|) <= tol for every real pair, computed on the host with scipy.sparse from
    the caller's CSR arrays and the eigenvectors EPSGetEigenpair returned (no device kernel involved)."""
    m = res["nconv"]
    real = res["eigi"][:m] == 0.0
    if not real.any():
        return
    r_a, _ = verify.residuals(csr, res["eigr"][:m][real], res["X"][:, :m][:, real])
    assert r_a.max() <= tol, r_a


def host_orth(res):
    """||X^T X - I||_max of the returned eigenvectors, in numpy."""
    return verify.orthogonality(res["X"][:, :res["nconv"]])


def matgen_norm_inf(csr):
    rp, ci, va = csr
    return max(np.add.reduceat(np.abs(va), rp[:-1])) if va.size else 0.0


def test_config1_laplacian_100(lib, orc):
    csr = matgen.laplacian_2d(100)
    v0 = matgen.start_vector(10000, 1)
    res = run(csr, hermitian=True, which="LM", nev=10, ncv=32, tol=1e-8, v0=v0)
    ref = orc.solve(*csr, hermitian=True, which="LM", nev=10, ncv=32, tol=1e-8, v0=v0)
    assert res["reason"] == 1 and res["nconv"] >= 10
    exact = matgen.laplacian_eigenvalues([100, 100])
    assert rel_match(res["eigr"], exact, 1e-10)
    # every distinct eigenvalue the oracle found among the wanted ones is found on the GPU
    for lam in np.unique(np.round(ref.eigr[:10], 9)):
        assert np.min(np.abs(res["eigr"] - lam)) / abs(lam) <= 1e-9
    check_residuals(csr, res, 1e-8)
    assert host_orth(res) <= 1e-12


def test_ex2_golden_on_gpu(lib):
    g = G["ex2_1"]
    csr = matgen.laplacian_2d(*g["grid"])
    res = run(csr, hermitian=True, which="LM", nev=g["nev"], ncv=g["ncv"], tol=1e-8,
              v0=matgen.start_vector(72 * 72, 1))
    got = np.unique(np.round(res["eigr"], 5))[::-1]
    assert list(got[:4]) == g["eigenvalues"]


@pytest.mark.parametrize("lock", [True, False])
def test_test2_goldens_on_gpu(lib, lock):
    g = G["test2_1"]
    csr = matgen.laplacian_1d(g["n"])
    for which, name in (("LR", "largest"), ("SR", "smallest")):
        A = sg.Mat(*csr)
        eps = sg.EPS().create()
        eps.setOperators(A)
        eps.setProblemType(sg.EPS.ProblemType.HEP)
        eps.setDimensions(g["nev"])
        eps.setTolerances(g["tol"])
        eps.setWhichEigenpairs(which)
        eps.setKrylovSchurLocking(lock)
        eps.setInitialSpace(matgen.start_vector(g["n"], 1))
        eps.solve()
        assert eps.getConvergedReason() == 1
        vals = [round(eps.getEigenvalue(i), 5) for i in range(g["nev"])]
        assert vals == g[name]


@pytest.mark.parametrize("arith", ["pair", "f64"])
def test_lap3d_parity(lib, orc, arith):
    m = 16
    csr = matgen.laplacian_3d(m)
    v0 = matgen.start_vector(m ** 3, 2)
    res = run(csr, hermitian=True, which="LR", nev=20, ncv=48, tol=1e-10, v0=v0, arith=arith)
    ref = orc.solve(*csr, hermitian=True, which="LR", nev=20, ncv=48, tol=1e-10, v0=v0)
    assert res["reason"] == 1 and res["nconv"] >= 20
    exact = matgen.laplacian_eigenvalues([m, m, m])
    assert rel_match(res["eigr"], exact, 1e-10)
    assert rel_match(res["eigr"][:20], ref.eigr, 1e-10) or rel_match(res["eigr"][:20], exact, 1e-12)
    check_residuals(csr, res, 1e-10)
    assert host_orth(res) <= 1e-12


@pytest.mark.parametrize("case", ["lap3d16", "lap2d_37x41", "lap3d24_ncv143", "lap3d64"])
def test_integer_gram_schmidt_parity(lib, case):
    """EPS_GB300_GS_INTEGER (every Gram-Schmidt product exact on the integer pipes) against the closed-form spectrum
    (1e-10), host-side residuals and orthogonality, and the FP64-FMA kernels: the same eigenvalues (1e-12, both
    ways) and about the same restart count.  The cases cover an odd row count, the widest basis the kernels take
    (143 columns) and more 512-row chunks than SMs."""
    dims, nev, ncv = {"lap3d16": ([16] * 3, 20, 48), "lap2d_37x41": ([37, 41], 12, 40),
                      "lap3d24_ncv143": ([24] * 3, 70, 143), "lap3d64": ([64] * 3, 20, 48)}[case]
    csr = matgen.laplacian_3d(dims[0]) if len(dims) == 3 else matgen.laplacian_2d(*dims)
    n = int(np.prod(dims))
    kw = dict(hermitian=True, which="LR", nev=nev, ncv=ncv, tol=1e-10, v0=matgen.start_vector(n, 3), arith="f64")
    a = run(csr, gs="integer", **kw)
    b = run(csr, gs="fma", **kw)
    assert a["stats"]["gs_exact"] == 1 and b["stats"]["gs_exact"] == 0
    assert a["reason"] == 1 and a["nconv"] >= nev
    exact = matgen.laplacian_eigenvalues(dims)
    assert rel_match(a["eigr"], exact, 1e-10)
    check_residuals(csr, a, 1e-10)
    assert host_orth(a) <= 1e-12
    assert rel_match(a["eigr"][:nev], b["eigr"][:b["nconv"]], 1e-12)
    assert rel_match(b["eigr"][:nev], a["eigr"][:a["nconv"]], 1e-12)
    assert abs(a["its"] - b["its"]) <= max(2, b["its"] // 10)


def test_brusselator_golden_on_gpu(lib, orc):
    g = G["ex9_1"]
    csr = matgen.brusselator(g["N"])
    res = run(csr, hermitian=False, which="LR", nev=g["nev"], tol=1e-8, v0=matgen.start_vector(100, 1))
    assert res["reason"] == 1
    got = [[round(a, 5), round(b, 5)] for a, b in zip(res["eigr"][:4], res["eigi"][:4])]
    assert got == g["eigenvalues"]
    dense = np.linalg.eigvals(matgen.csr_to_dense(*csr))
    for a, b in zip(res["eigr"], res["eigi"]):
        z = complex(a, b)
        assert np.min(np.abs(dense - z)) / abs(z) < 1e-9
    # residuals of the complex pairs through EPSComputeError
    for i in range(res["nconv"]):
        assert res["errors"][i] < 1e-7


def test_rdb200_from_petsc_file_on_gpu(lib, orc, tmp_path):
    """The reference's real non-symmetric matrix, written in PETSc's binary format and read back by MatLoad, solved
    as ex4 does (EPS_NHEP, largest magnitude, nev 4, tol 1e-8): the digits of ex4_1.out; then at tol 1e-10 against
    the oracle and a dense solve."""
    g = G["ex4_1"]
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "rdb200.npz"))
    path = str(tmp_path / "rdb200.petsc")
    sg.Mat(d["rowptr"], d["colidx"], d["vals"]).save(path)
    A = sg.Mat.load(path)
    csr = (A.rowptr, A.colidx, A.vals)
    v0 = matgen.start_vector(200, 1)
    res = run(csr, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"], v0=v0)
    assert res["reason"] == 1
    assert [round(v, 5) for v in res["eigr"][:4]] == g["eigenvalues"]
    res = run(csr, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-10, v0=v0)
    ref = orc.solve(*csr, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-10, v0=v0)
    assert res["reason"] == 1 and ref.reason == 1
    dense = np.linalg.eigvals(matgen.csr_to_dense(*csr))
    for i in range(4):  # both stop at estimates below 1e-10; the eigenvalues agree within a few times that
        assert abs(res["eigr"][i] - ref.eigr[i]) <= 1e-9 * abs(ref.eigr[i])
        assert np.min(np.abs(dense - res["eigr"][i])) <= 1e-10 * abs(res["eigr"][i])
    check_residuals(csr, res, 1e-10)


def test_convdiff_nhep_parity(lib, orc):
    N, Pe = 40, 10.0
    csr = matgen.convection_diffusion_2d(N, Pe)
    v0 = matgen.start_vector(N * N, 3)
    res = run(csr, hermitian=False, which="LR", nev=10, ncv=40, tol=1e-12, v0=v0)
    assert res["reason"] == 1 and res["nconv"] >= 10
    exact = matgen.convdiff_eigenvalues(N, Pe)
    assert rel_match(res["eigr"], exact, 1e-10)
    # the spectrum is real but doubly degenerate (lambda(i, j) = lambda(j, i)) and the operator strongly non-normal:
    # rounding may turn a degenerate pair into a conjugate pair with tiny imaginary parts
    assert np.all(np.abs(res["eigi"]) <= 1e-9 * np.abs(res["eigr"]))
    ref = orc.solve(*csr, hermitian=False, which="LR", nev=10, ncv=40, tol=1e-12, v0=v0)
    assert rel_match(res["eigr"][:10], ref.eigr, 1e-10)
    check_residuals(csr, res, 1e-10)


def test_zero_start_vector_error(lib):
    csr = matgen.laplacian_1d(50)
    with pytest.raises(sg.SlepcError) as ei:
        run(csr, hermitian=True, nev=2, v0=np.zeros(50))
    assert ei.value.code == 77


def test_repeatable(lib):
    csr = matgen.laplacian_2d(40)
    v0 = matgen.start_vector(1600, 5)
    a = run(csr, hermitian=True, which="LR", nev=8, ncv=24, tol=1e-10, v0=v0)
    b = run(csr, hermitian=True, which="LR", nev=8, ncv=24, tol=1e-10, v0=v0)
    assert np.array_equal(a["eigr"], b["eigr"])
    assert np.array_equal(a["X"], b["X"])


@pytest.mark.parametrize("tol", [1e-10, 1e-5])
def test_precision_form(lib, orc, tol):
    """FP32 values and basis with pair accumulation; the FP64 recheck passes at tol 1e-5 (no sweep) and fails at
    1e-10, where the FP64-class refinement sweep finishes.  Error against the FP64 oracle stated per eigenpair."""
    m = 14
    csr = matgen.laplacian_3d_randdiag(m, 13)
    v0 = matgen.start_vector(m ** 3, 6)
    nev = 12
    res = run(csr, hermitian=True, which="LR", nev=nev, ncv=40, tol=tol, v0=v0, arith="f32")
    st = res["eps"].getStats()
    assert res["reason"] == 1 and res["nconv"] >= nev
    assert st["precision_steps"] > 0
    if tol < 1e-6:
        assert st["krylov_steps"] > st["precision_steps"]  # the refinement sweep ran
    else:
        assert st["krylov_steps"] == st["precision_steps"]
    dense = np.linalg.eigvalsh(matgen.csr_to_dense(*csr))
    errs = [np.min(np.abs(dense - v)) / abs(v) for v in res["eigr"][:nev]]
    assert max(errs) <= max(tol, 1e-10), errs  # per-eigenpair error against the FP64 dense solve
    check_residuals(csr, res, tol)
    assert host_orth(res) <= (1e-12 if tol < 1e-6 else 1e-6)


@pytest.mark.parametrize("herm", [True, False])
def test_tensor_restart_matches_pair_restart(lib, herm):
    """The bf16 tensor-core restart (error-free split) against the CUDA-core pair-arithmetic restart: the same
    eigenvalues to 1e-12, residuals within tol, and a basis orthonormal to 1e-12 after every restart."""
    if herm:
        csr, kw = matgen.laplacian_3d_randdiag(18, 3), dict(hermitian=True, which="LR", nev=16, ncv=56)
    else:
        csr, kw = matgen.convection_diffusion_2d(40, 2.0), dict(hermitian=False, which="LR", nev=10, ncv=40)
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 21)
    a = run(csr, tol=1e-10, v0=v0, restart="tensor", **kw)
    b = run(csr, tol=1e-10, v0=v0, restart="pair", **kw)
    for r in (a, b):
        assert r["reason"] == 1 and r["nconv"] >= kw["nev"]
        check_residuals(csr, r, 1e-10)
        if herm:
            assert host_orth(r) <= 1e-12
    # symmetric: 1e-12.  The convection-diffusion operator (mildly non-normal at Pe = 2) has doubly degenerate
    # eigenvalues whose computed copies move with the rounding; 1e-10 is the parity bound of the closed form.
    agree = 1e-12 if herm else 1e-10
    vb = np.asarray(b["eigr"]) + 1j * np.asarray(b["eigi"])
    for x, y in zip(a["eigr"][:kw["nev"]], a["eigi"][:kw["nev"]]):
        z = complex(x, y)
        assert np.min(np.abs(vb - z)) / abs(z) <= agree


@pytest.mark.parametrize("case", ["lap3d_wide", "lap3d_narrow", "convdiff"])
def test_tcgen05_restart_is_bit_identical(lib, case):
    """The restart on tcgen05 (TMEM accumulators) against the same error-free split on mma.sync: every level sum is
    exact in FP32, so whole solves agree bit for bit (eigenvalues, restart counts, eigenvectors).  The cases cover
    output chunks wider than 64 columns (two TMEM passes), a last K stage of 16, row counts that are not multiples
    of the 128-row tile, and the non-symmetric solver."""
    if case == "lap3d_wide":
        csr, kw = matgen.laplacian_3d_randdiag(30, 3), dict(hermitian=True, which="LR", nev=40, ncv=110)
    elif case == "lap3d_narrow":
        csr, kw = matgen.laplacian_3d_randdiag(23, 5), dict(hermitian=True, which="LR", nev=12, ncv=40)
    else:
        csr, kw = matgen.convection_diffusion_2d(45, 2.0), dict(hermitian=False, which="LR", nev=10, ncv=40)
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 21)
    a = run(csr, tol=1e-10, v0=v0, restart="tcgen05", **kw)
    b = run(csr, tol=1e-10, v0=v0, restart="mma_sync", **kw)
    assert a["reason"] == 1 and b["reason"] == 1
    assert a["its"] == b["its"] and a["nconv"] == b["nconv"]
    assert np.array_equal(a["eigr"], b["eigr"]) and np.array_equal(a["eigi"], b["eigi"])
    assert np.array_equal(a["X"], b["X"])


@pytest.mark.parametrize("case", ["lap3d_wide", "lap3d_narrow", "convdiff"])
def test_tcgen05_restart_fp64_storage(lib, case):
    """The tcgen05 restart on IEEE-double storage (Q in 8 slices for K <= 128, exact level sums rounded once to a
    double) against the CUDA-core FP64 FMA restart: the same eigenvalues to 1e-12, both at 1e-10 against the closed
    form where there is one, host-side residuals at tol and orthonormal eigenvectors.  The wide case has K up to 110
    and two output chunks; the narrow one a last K stage of 16."""
    if case == "lap3d_wide":
        csr, kw = matgen.laplacian_3d(30), dict(hermitian=True, which="LR", nev=40, ncv=110)
        exact = matgen.laplacian_eigenvalues([30, 30, 30])
    elif case == "lap3d_narrow":
        csr, kw = matgen.laplacian_3d_randdiag(23, 5), dict(hermitian=True, which="LR", nev=12, ncv=40)
        exact = None
    else:
        csr, kw = matgen.convection_diffusion_2d(45, 2.0), dict(hermitian=False, which="LR", nev=10, ncv=40)
        exact = matgen.convdiff_eigenvalues(45, 2.0)
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 21)
    a = run(csr, tol=1e-10, v0=v0, arith="f64", restart="tcgen05", **kw)
    b = run(csr, tol=1e-10, v0=v0, arith="f64", restart="pair", **kw)
    assert a["reason"] == 1 and b["reason"] == 1 and a["nconv"] >= kw["nev"]
    # set-based: a degenerate spectrum may converge different numbers of copies; the non-normal convection-diffusion
    # operator's Ritz values are sensitive at the level of its tolerance, so that case uses the parity bound 1e-10
    agree = 1e-12 if kw["hermitian"] else 1e-10
    for x, y in ((a, b), (b, a)):
        for v in x["eigr"][:kw["nev"]]:
            assert np.min(np.abs(y["eigr"][:y["nconv"]] - v)) / abs(v) <= agree
    if exact is not None:
        assert rel_match(a["eigr"][:a["nconv"]], exact, 1e-10)
    check_residuals(csr, a, 1e-10)
    if kw["hermitian"]:
        assert host_orth(a) <= 1e-12


@pytest.mark.parametrize("lock", [True, False])
def test_test2_interior_harmonic_golden_on_gpu(lib, lock):
    """test2.c's third solve on the device: harmonic extraction for the eigenvalues closest to 2.1."""
    g = G["test2_1"]
    csr = matgen.laplacian_1d(g["n"])
    res = run(csr, hermitian=True, which="TM", nev=g["nev"], tol=g["tol"], v0=matgen.start_vector(g["n"], 1),
              harmonic=True, target=g["target"], lock=lock)
    assert res["reason"] == 1
    assert [round(v, 5) for v in res["eigr"][:4]] == g["interior"]
    assert res["eps"].getExtraction() == 1 and res["eps"].getTarget() == g["target"]


@pytest.mark.parametrize("arith", ["pair", "f64"])
def test_harmonic_hep_parity(lib, orc, arith):
    n, tgt = 400, 1.0
    csr = matgen.laplacian_1d(n)
    v0 = matgen.start_vector(n, 1)
    kw = dict(hermitian=True, which="TM", nev=4, ncv=30, tol=1e-10, v0=v0, harmonic=True, target=tgt)
    res = run(csr, arith=arith, **kw)
    ref = orc.solve(*csr, **kw)
    assert res["reason"] == 1 and ref.reason == 1
    ex = 2 - 2 * np.cos(np.arange(1, n + 1) * np.pi / (n + 1))
    want = ex[np.argsort(np.abs(ex - tgt))][:4]
    got = np.asarray(res["eigr"][:4])
    assert np.max(np.abs(got - want) / want) <= 1e-10
    assert np.max(np.abs(got - np.asarray(ref.eigr[:4])) / want) <= 1e-10
    assert np.all(np.abs(got[:-1] - tgt) <= np.abs(got[1:] - tgt))  # nearest to the target first
    check_residuals(csr, res, 1e-10)
    assert host_orth(res) <= 1e-12


def test_harmonic_nhep_parity(lib, orc):
    N, Pe, tgt = 20, 2.0, 4.0
    csr = matgen.convection_diffusion_2d(N, Pe)
    v0 = matgen.start_vector(N * N, 3)
    kw = dict(hermitian=False, which="TM", nev=4, ncv=30, tol=1e-10, v0=v0, harmonic=True, target=tgt)
    res = run(csr, **kw)
    ref = orc.solve(*csr, **kw)
    assert res["reason"] == 1 and ref.reason == 1
    ex = matgen.convdiff_eigenvalues(N, Pe)
    for v in res["eigr"][:4]:
        assert np.min(np.abs(ex - v)) <= 1e-10 * abs(v)
        assert np.min(np.abs(np.asarray(ref.eigr[:4]) - v)) <= 1e-10 * abs(v)
    assert np.max(np.abs(res["eigi"][:4])) == 0.0


@pytest.mark.parametrize("ds", ["refined", "qr"])
def test_ritz_target_criterion(lib, ds):
    """EPS_TARGET_MAGNITUDE with Ritz extraction orders by distance to the target in both symmetric projected
    solvers: a target below the spectrum selects the smallest eigenvalues, nearest first."""
    n = 100
    csr = matgen.laplacian_1d(n)
    res = run(csr, hermitian=True, which="TM", nev=4, ncv=20, tol=1e-10, v0=matgen.start_vector(n, 1), target=-0.5,
              ds=ds)
    assert res["reason"] == 1
    ex = np.sort(2 - 2 * np.cos(np.arange(1, n + 1) * np.pi / (n + 1)))[:4]
    assert np.max(np.abs(np.asarray(res["eigr"][:4]) - ex) / ex) <= 1e-10


def test_batch_rejects_targets(lib):
    csr = matgen.laplacian_1d(200)
    A = sg.Mat(*csr)
    eps = sg.EPS().create()
    eps.setOperators(A)
    eps.setProblemType(sg.EPS.ProblemType.HEP)
    eps.setDimensions(4, 20)
    eps.setWhichEigenpairs("TM")
    eps.setTarget(1.0)
    eps.setExtraction("harmonic")
    with pytest.raises(sg.SlepcError) as e:
        sg.solve_batch([eps])
    assert e.value.code == 56  # PETSC_ERR_SUP


def test_error_view_prints_the_reference_text(lib, tmp_path):
    """EPSErrorView's default report (epsview.c:297-333) against the lines the reference's tests printed: ex2
    (symmetric), ex9 (complex pairs: 0.00007+2.13946i), ex4 (rdb200 read by MatLoad), and test2's three solves
    (largest, smallest, harmonic interior around 2.1).  The INFO_DETAIL table and EPSConvergedReasonView follow
    the reference's layout."""
    cases = []
    g = G["ex2_1"]
    cases.append((matgen.laplacian_2d(*g["grid"]), dict(hermitian=True, which="LM", nev=4, ncv=20, tol=1e-8),
                  g["errorview"][0]))
    g = G["ex9_1"]
    cases.append((matgen.brusselator(g["N"]), dict(hermitian=False, which="LR", nev=4, tol=1e-8), g["errorview"][0]))
    g = G["ex4_1"]
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "rdb200.npz"))
    path = str(tmp_path / "rdb200.petsc")
    sg.Mat(d["rowptr"], d["colidx"], d["vals"]).save(path)
    A = sg.Mat.load(path)
    cases.append(((A.rowptr, A.colidx, A.vals), dict(hermitian=False, which="LM", nev=4, tol=1e-8),
                  g["errorview"][0]))
    g = G["test2_1"]
    lap = matgen.laplacian_1d(g["n"])
    for kw, want in ((dict(which="LR"), g["errorview"][0]), (dict(which="SR"), g["errorview"][1]),
                     (dict(which="TM", harmonic=True, target=g["target"]), g["errorview"][2])):
        cases.append((lap, dict(hermitian=True, nev=4, tol=g["tol"], **kw), want))
    for csr, kw, want in cases:
        n = len(csr[0]) - 1
        res = run(csr, v0=matgen.start_vector(n, 1), **kw)
        eps = res["eps"]
        text = eps.errorView()
        assert text.splitlines()[:2] == want, (text, want)
        assert text.endswith("\n\n")
        nconv = eps.getConverged()
        assert eps.convergedReasonView() == (f" Linear eigensolve converged ({nconv} eigenpairs) due to "
                                             f"CONVERGED_TOL; iterations {eps.getIterationNumber()}\n")
        detail = eps.errorView(detail=True).splitlines()
        sep = " ---------------------- --------------------"
        assert detail[0] == sep and detail[2] == sep and detail[-1] == sep
        assert detail[1] == "            k             ||Ax-kx||/||kx||"
        assert len(detail) == nconv + 4
        for i, line in enumerate(detail[3:-1]):
            z = complex(eps.getEigenvalue(i))
            kr, ki = z.real, z.imag
            err = eps.computeError(i)
            want_line = (f"  {kr: 9f}{ki:+9f}i      {err:12g}" if ki != 0.0 else f"    {kr: 12f}           {err:12g}")
            assert line == want_line
        values = eps.valuesView().splitlines()
        assert values[0] == "Eigenvalues = " and len(values) == nconv + 2 and values[-1] == ""
        assert values[1] == "   " + want[1].split(",")[0].strip()


def test_monitor_and_matlab_values_test23(lib, orc, tmp_path):
    """test23.c TEST 2 on the device: diag(1..20), -eps_largest_real -eps_monitor -eps_view_values ::ascii_matlab
    given as options.  The monitor lines, after the test's own filter of the error estimates, are the reference's
    two lines; the restart-by-restart values follow the oracle's monitor; the MATLAB values report is the
    reference's."""
    g = G["test23_2"]
    n = g["n"]
    rp, ci, va = np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.arange(1, n + 1, dtype=float)
    v0 = matgen.start_vector(n, 1)
    mon, val = tmp_path / "mon.txt", tmp_path / "val.txt"
    sg.initialize(["test23", "-eps_largest_real", "-eps_monitor", ":" + str(mon),
                   "-eps_view_values", ":" + str(val) + ":ascii_matlab"])
    try:
        A = sg.Mat(rp, ci, va)
        eps = sg.EPS().create()
        eps.setOperators(A)
        eps.setName("eps")
        eps.setFromOptions()
        eps.setInitialSpace(v0)
        seen = []
        eps.monitorSet(lambda its, nconv, er, ei, es: seen.append((its, nconv, er.copy(), es.copy())))
        eps.solve()
        assert eps.getConvergedReason() == 1
    finally:
        sg.initialize(["prog"])
    lines = mon.read_text().splitlines()
    assert [re.sub(r"[0-9]\.[0-9]*e-([0-9]*)", "removed", l) for l in lines] == g["monitor"]
    ref = []
    r = orc.solve(rp, ci, va, hermitian=False, which="LR", nev=1, tol=1e-8, v0=v0,
                  monitor=lambda its, nconv, er, ei, es, nest: ref.append((its, nconv, list(er), list(es))))
    assert r.reason == 1 and len(seen) == len(ref) == eps.getIterationNumber()
    for (its, k, er, es), (its_r, k_r, er_r, es_r) in zip(seen, ref):
        assert its == its_r and k == k_r and len(er) == len(er_r)
        assert np.allclose(er, er_r, rtol=1e-9, atol=0)
    vals = [l.strip() for l in val.read_text().splitlines()]
    fixed = [re.sub(r"^(2\.[0-9]*e\+01|1\.9999999999[0-9]*e\+01)$", "2.0000000000000000e+01", l) for l in vals]
    assert fixed == g["values_matlab"]


@pytest.mark.parametrize("lock", [True, False])
def test_ex5_markov_golden_on_gpu(lib, orc, lock):
    """ex5.c on the device: the Markov random walk (n = 120), non-Hermitian, largest real, nev 4: the digits of
    ex5_1.out (after its filter), the EPSErrorView line, and the oracle's eigenvalues to 1e-10 at tol 1e-10."""
    g = G["ex5_1"]
    csr = matgen.markov_walk(g["m"])
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 1)
    res = run(csr, hermitian=False, which=g["which"], nev=g["nev"], tol=g["tol"], lock=lock, v0=v0)
    assert res["reason"] == 1
    got = [f"{v:.5f}" for v in res["eigr"][:4]]
    for a, b in g["filter"]:
        got = [b if x == a else x for x in got]
    assert [float(x) for x in got] == g["eigenvalues"]
    text = res["eps"].errorView().splitlines()[:2]
    for a, b in g["filter"]:
        text = [t.replace(a, b) for t in text]
    assert text == g["errorview"][0]
    res = run(csr, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-10, lock=lock, v0=v0)
    ref = orc.solve(*csr, hermitian=False, which=g["which"], nev=g["nev"], tol=1e-10, lock=lock, v0=v0)
    assert ref.reason == 1
    for i in range(4):  # both stop at estimates below 1e-10; the eigenvalues agree within a few times that
        assert abs(res["eigr"][i] - ref.eigr[i]) <= 1e-9 * abs(ref.eigr[i])


@pytest.mark.parametrize("key,gen", [("test4_1", "lap1d"), ("test6_1", "diag")])
def test_test4_test6_goldens_on_gpu(lib, key, gen):
    """test4.c and test6.c on the device: HEP, nev 4, largest magnitude; digits and the EPSErrorView line."""
    g = G[key]
    n = g["n"]
    csr = matgen.laplacian_1d(n) if gen == "lap1d" else matgen.diagonal(np.arange(1, n + 1, dtype=float))
    res = run(csr, hermitian=True, which=g["which"], nev=g["nev"], tol=g["tol"], v0=matgen.start_vector(n, 1))
    assert res["reason"] == 1
    assert [round(v, 5) for v in res["eigr"][:4]] == g["eigenvalues"]
    assert res["eps"].errorView().splitlines()[:2] == g["errorview"][0]


@pytest.mark.parametrize("arith", ["pair", "f64"])
@pytest.mark.parametrize("kind", ["hep", "nhep", "ghep"])
def test_device_eigenvectors_match_getEigenpair(lib, arith, kind):
    """EPSGB300GetDeviceEigenvectors: IEEE doubles in EPSGetEigenpair order whatever the storage format; a complex
    pair occupies two columns (real part, imaginary part)."""
    B = None
    if kind == "hep":
        csr, kw = matgen.laplacian_3d_randdiag(14, 3), dict(hermitian=True, which="LR", nev=8, ncv=32)
    elif kind == "nhep":
        csr, kw = matgen.brusselator(50), dict(hermitian=False, which="LR", nev=6, ncv=24)
    else:
        csr, kw = matgen.laplacian_2d(20), dict(hermitian=True, which="LR", nev=6, ncv=24)
        B = matgen.diagonal(2.0 / np.log(np.arange(400) + 2.0))
    n = len(csr[0]) - 1
    res = run(csr, tol=1e-10, v0=matgen.start_vector(n, 5), arith=arith, B=B, **kw)
    eps, m = res["eps"], res["nconv"]
    assert m >= kw["nev"]
    Xd = eps.copyDeviceEigenvectors()
    assert Xd.shape == (n, m) and Xd.dtype == np.float64
    vr, vi = np.zeros(n), np.zeros(n)
    saw_pair = False
    for i in range(m):
        lam = eps.getEigenpair(i, vr, vi)
        scale = max(1.0, np.abs(vr).max())
        if isinstance(lam, complex) and lam.imag > 0 and i + 1 < m:
            saw_pair = True
            assert np.allclose(Xd[:, i], vr, rtol=0, atol=1e-15 * scale)
            assert np.allclose(Xd[:, i + 1], vi, rtol=0, atol=1e-15 * scale)
        elif not isinstance(lam, complex):
            assert np.allclose(Xd[:, i], vr, rtol=0, atol=1e-15 * scale)
    if kind == "nhep":
        assert saw_pair  # the Brusselator's wanted eigenvalues are complex pairs
    # the array is refreshed by the next solve
    eps.solve()
    assert np.allclose(eps.copyDeviceEigenvectors()[:, 0], Xd[:, 0], rtol=0, atol=1e-12)


@pytest.mark.parametrize("arith", ["f64", "pair"])
def test_test20_full_basis_on_gpu(lib, arith):
    """test20.c: the smallest eigenvalue of the 1-D Laplacian n = 18 with the default ncv (16) and with ncv = 18 = n,
    a full basis whose last factorisation step ends in a breakdown (beta = 0) with every Ritz value converged; ncv
    above n is clamped to n (epssetup.c:336-337)."""
    g = G["test20_1"]
    n = g["n"]
    csr = matgen.laplacian_1d(n)
    for ncv, want in zip(g["ncv"], g["eigenvalues"]):
        res = run(csr, hermitian=True, which=g["which"], nev=g["nev"], ncv=ncv, tol=g["tol"],
                  v0=matgen.start_vector(n, 1), arith=arith)
        assert res["reason"] == 1 and res["nconv"] >= 1
        assert round(float(res["eigr"][0]), 5) == want
        check_residuals(csr, res, g["tol"])
    res = run(csr, hermitian=True, which="SR", nev=2, ncv=40, tol=g["tol"], v0=matgen.start_vector(n, 1),
              arith=arith)
    assert res["reason"] == 1 and res["eps"].getDimensions()[1] == n


def test_full_basis_every_eigenpair(lib):
    """ncv = nev = n: one restart gives the whole spectrum (HEP against LAPACK's eigh; NHEP against eigvals of a
    dense non-normal matrix with complex pairs)."""
    import scipy.linalg as sl

    csr = matgen.laplacian_3d_randdiag(4, 2)  # n = 64, distinct eigenvalues
    n = len(csr[0]) - 1
    res = run(csr, hermitian=True, which="LR", nev=n, ncv=n, tol=1e-12, v0=matgen.start_vector(n, 2), arith="f64")
    assert res["reason"] == 1 and res["nconv"] == n and res["its"] == 1
    w = sl.eigh(matgen.csr_to_dense(*csr), eigvals_only=True)
    assert np.max(np.abs(np.sort(res["eigr"]) - np.sort(w))) <= 1e-12 * np.max(np.abs(w))
    check_residuals(csr, res, 1e-12)
    assert host_orth(res) <= 1e-12
    # non-Hermitian: the Brusselator at n = 40 (complex pairs), all eigenvalues
    csr = matgen.brusselator(20)
    n = len(csr[0]) - 1
    res = run(csr, hermitian=False, which="LM", nev=n, ncv=n, tol=1e-12, v0=matgen.start_vector(n, 2), arith="f64")
    assert res["reason"] == 1 and res["nconv"] == n
    w = np.linalg.eigvals(matgen.csr_to_dense(*csr))
    got = res["eigr"] + 1j * res["eigi"]
    for lam in w:
        assert np.min(np.abs(got - lam)) <= 1e-10 * np.max(np.abs(w)), lam


@pytest.mark.parametrize("arith,ds", [("f64", "qr"), ("pair", "qr"), ("f64", "refined")])
def test_wide_basis_nev100_default_ncv(lib, arith, ds):
    """nev = 100 with the default ncv = 2 nev = 200 (EPSSetDimensions_Default, epssetup.c:663): a projected problem
    of 201 rows, past the shared-memory solver (Q rotated in place), the column-group Gram-Schmidt and the wide
    restart.  The 3-D Laplacian 32^3's closed-form spectrum, host residuals and orthogonality."""
    csr = matgen.laplacian_3d(32)
    n = 32 ** 3
    res = run(csr, hermitian=True, which="LR", nev=100, tol=1e-10, v0=matgen.start_vector(n, 7), arith=arith, ds=ds)
    assert res["eps"].getDimensions()[1] == 200
    assert res["reason"] == 1 and res["nconv"] >= 100
    m = verify.match_spectrum(res["eigr"][:res["nconv"]], matgen.laplacian_eigenvalues([32, 32, 32]), "LR", 100)
    assert m["ok"], m
    check_residuals(csr, res, 1e-10)
    assert host_orth(res) <= 1e-12


def test_wide_basis_nev500(lib):
    """nev = 500: the default ncv is nev + mpd = 1000 with mpd = 500 (epssetup.c:664-667), a projected problem of
    1001 rows.  The 2-D Laplacian 120 x 97 against its closed form."""
    csr = matgen.laplacian_2d(120, 97)
    n = 120 * 97
    res = run(csr, hermitian=True, which="SR", nev=500, tol=1e-9, v0=matgen.start_vector(n, 8), arith="f64")
    assert res["eps"].getDimensions() == (500, 1000, 500)
    assert res["reason"] == 1 and res["nconv"] >= 500
    m = verify.match_spectrum(res["eigr"][:res["nconv"]], matgen.laplacian_eigenvalues([120, 97]), "SR", 500,
                              rel_tol=1e-9)
    assert m["ok"], m
    check_residuals(csr, res, 1e-9)
    assert host_orth(res) <= 1e-12


def test_wide_basis_nonsymmetric(lib):
    """NHEP with nev = 100 and the default ncv = 200: the non-symmetric projected solver in place in the EPS's arrays
    (201 rows).  Convection-diffusion 40^2 at Pe = 1 (the similarity to a symmetric matrix is well conditioned, so
    the closed form pins the eigenvalues to 1e-9); ncv above 639 is PETSC_ERR_SUP at setup."""
    N, pe = 40, 1.0
    csr = matgen.convection_diffusion_2d(N, pe)
    n = N * N
    res = run(csr, hermitian=False, which="LR", nev=100, tol=1e-10, v0=matgen.start_vector(n, 9), arith="f64")
    assert res["eps"].getDimensions()[1] == 200
    assert res["reason"] == 1 and res["nconv"] >= 100
    k = res["nconv"]
    assert np.max(np.abs(res["eigi"][:k])) <= 1e-9 * np.max(np.abs(res["eigr"][:k]))
    m = verify.match_spectrum(res["eigr"][:k], matgen.convdiff_eigenvalues(N, pe), "LR", 100, rel_tol=1e-9)
    assert m["ok"], m
    check_residuals(csr, res, 1e-10)
    with pytest.raises(sg.SlepcError) as e:
        run(matgen.convection_diffusion_2d(30, pe), hermitian=False, which="LR", nev=10, ncv=700, tol=1e-8)
    assert e.value.code == 56


@pytest.mark.parametrize("arith,herm", [("f64", True), ("pair", True), ("f64", False)])
def test_graph_segments_match_direct_launches(lib, arith, herm):
    """Factorisation segments replayed from captured CUDA graphs give the same bits as direct launches: three
    solves with graphs on (the second and third replay the segments seen before) against one with them off.  The
    Gram-Schmidt method is fixed (FP64 FMA for IEEE-double storage): the automatic choice differs between the two
    launch modes."""
    if herm:
        csr, kw = matgen.laplacian_2d(100), dict(hermitian=True, which="LM", nev=10, ncv=32)
    else:
        csr, kw = matgen.convection_diffusion_2d(60, 10.0), dict(hermitian=False, which="LR", nev=8, ncv=32)
    n = len(csr[0]) - 1
    A = sg.Mat(*csr)

    def make(mode):
        e = sg.EPS().create()
        e.setOperators(A)
        e.setProblemType(sg.EPS.ProblemType.HEP if kw["hermitian"] else sg.EPS.ProblemType.NHEP)
        e.setDimensions(kw["nev"], kw["ncv"])
        e.setTolerances(1e-10)
        e.setWhichEigenpairs(kw["which"])
        e.setArithmetic(arith)
        e.setGSMethod("fma")
        e.setGraphCapture(mode)
        e.setInitialSpace(matgen.start_vector(n, 4))
        return e

    def vals(e):
        k = e.getConverged()
        return np.array([complex(e.getEigenvalue(i)) for i in range(k)]), e.getIterationNumber()

    ref = make(0)
    ref.solve()
    want = vals(ref)
    assert ref.getStats()["graph_segments"] == 0
    e = make(1)
    replays = []
    for _ in range(3):
        e.solve()
        got = vals(e)
        assert got[1] == want[1] and np.array_equal(got[0], want[0])
        replays.append(e.getStats()["graph_segments"])
    assert replays[2] > 0 and replays[2] >= replays[0]


@pytest.mark.parametrize("arith", ["f64", "pair"])
def test_ex11_deflation_space_golden_on_gpu(lib, orc, arith):
    """ex11.c: the Fiedler vectors of a 10 x 10 mesh's graph Laplacian with the constant vector (its null space) as
    deflation space (EPSSetDeflationSpace): the eigenvalues ex11_1.out prints, every eigenvector orthogonal to the
    deflation space, and the oracle's deflated solve at 1e-10; without the space the zero eigenvalue comes first."""
    g = G["ex11_1"]
    csr = matgen.graph_laplacian_2d(*g["grid"])
    n = len(csr[0]) - 1
    v0 = matgen.start_vector(n, 1)
    res = run(csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=g["tol"], v0=v0, arith=arith,
              deflation=np.ones(n))
    assert res["reason"] == 1 and res["nconv"] >= g["nev"]
    assert [round(float(v), 5) for v in res["eigr"][:g["nev"]]] == g["eigenvalues"]
    X = res["X"][:, :res["nconv"]]
    assert np.abs(X.sum(axis=0)).max() < 1e-10 * np.sqrt(n)
    check_residuals(csr, res, 1e-8)
    ref = orc.solve(*csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=1e-12,
                    deflation=np.ones(n), v0=v0)
    tight = run(csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=1e-12, v0=v0, arith=arith,
                deflation=np.ones(n))
    assert rel_match(tight["eigr"][:g["nev"]], ref.eigr[:ref.nconv], 1e-10)
    plain = run(csr, hermitian=True, which=g["which"], nev=g["nev"], keep=g["keep"], tol=g["tol"], v0=v0, arith=arith)
    assert abs(plain["eigr"][0]) < 1e-8


def test_deflation_space_of_eigenvectors(lib):
    """Deflating the three lowest eigenvectors of a 1-D Laplacian (and a dependent fourth vector, which is dropped)
    leaves the next eigenvalues as the smallest ones found; the eigenvectors are orthogonal to the space. Harmonic
    extraction and generalised problems refuse a deflation space (PETSC_ERR_SUP)."""
    n = 400
    csr = matgen.laplacian_1d(n)
    exact = np.sort(matgen.laplacian_eigenvalues([n]))
    k = np.arange(1, n + 1)
    W = np.stack([np.sin(j * np.pi * k / (n + 1)) for j in (1, 2, 3)], axis=1)  # the three lowest eigenvectors
    W = np.concatenate([W, (W[:, :1] + 2.0 * W[:, 1:2])], axis=1)
    res = run(csr, hermitian=True, which="SR", nev=4, ncv=24, tol=1e-10, v0=matgen.start_vector(n, 2), arith="f64",
              deflation=W)
    assert res["reason"] == 1 and res["nconv"] >= 4
    assert np.max(np.abs(np.sort(res["eigr"][:4]) - exact[3:7]) / exact[3:7]) < 1e-10
    Q, _ = np.linalg.qr(W[:, :3])
    assert np.abs(Q.T @ res["X"][:, :res["nconv"]]).max() < 1e-10
    with pytest.raises(sg.SlepcError) as e:
        run(csr, hermitian=True, which="TM", target=0.1, harmonic=True, nev=2, ncv=20, deflation=W[:, :1])
    assert e.value.code == 56
    with pytest.raises(sg.SlepcError) as e:
        run(csr, hermitian=True, which="SR", nev=2, ncv=20, deflation=W[:, :1], B=matgen.diagonal(np.ones(n) * 2.0))
    assert e.value.code == 56
