"""ASCII viewers and the EPS text reports without a GPU: the format stack, PetscViewerASCIIPrintf, the stdout viewer,
EPSConvergedReasonView of an EPS that has not run (epsview.c:243-262 prints CONVERGED_ITERATING with 0 iterations),
EPSErrorView before EPSSolve (PETSC_ERR_ORDER) and binary calls on an ASCII viewer (PETSC_ERR_SUP).  The reports
of solved problems are checked against the reference's printed text in test_gpu_eps.py."""
import ctypes

import numpy as np
import pytest

import slepc_gb300 as sg

P = ctypes.c_void_p
PETSC_ERR_SUP, PETSC_ERR_ORDER = 56, 58
PETSC_VIEWER_DEFAULT, PETSC_VIEWER_ASCII_INFO_DETAIL = 0, 5


@pytest.fixture(scope="module")
def lib():
    sg.build()
    lib = sg.load()
    lib.PETSC_VIEWER_STDOUT_.restype = P
    lib.PETSC_VIEWER_STDOUT_.argtypes = [ctypes.c_int]
    lib.PetscViewerGetFormat.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    lib.PetscViewerASCIIGetStdout.argtypes = [ctypes.c_int, ctypes.POINTER(P)]
    lib.MatLoad.argtypes = [P, P]
    return lib


def open_ascii(lib, path):
    v = P()
    assert lib.PetscViewerASCIIOpen(0, str(path).encode(), ctypes.byref(v)) == 0
    return v


def test_format_stack_and_printf(lib, tmp_path):
    path = tmp_path / "out.txt"
    v = open_ascii(lib, path)
    fmt = ctypes.c_int(-1)
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT
    assert lib.PetscViewerPushFormat(v, PETSC_VIEWER_ASCII_INFO_DETAIL) == 0
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_ASCII_INFO_DETAIL
    assert lib.PetscViewerPopFormat(v) == 0
    assert lib.PetscViewerGetFormat(v, ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT
    assert lib.PetscViewerASCIIPrintf(v, b"n=%d x=%.3f\n", ctypes.c_int(30), ctypes.c_double(2.5)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0 and not v.value
    assert path.read_text() == "n=30 x=2.500\n"


def test_stdout_viewer_is_shared_and_not_closed(lib):
    a = lib.PETSC_VIEWER_STDOUT_(0)
    b = P()
    assert lib.PetscViewerASCIIGetStdout(1, ctypes.byref(b)) == 0
    assert a and a == b.value
    assert lib.PetscViewerDestroy(ctypes.byref(b)) == 0 and not b.value
    fmt = ctypes.c_int(-1)
    assert lib.PetscViewerGetFormat(P(a), ctypes.byref(fmt)) == 0 and fmt.value == PETSC_VIEWER_DEFAULT


def test_reports_before_solve(lib, tmp_path):
    eps = sg.EPS().create()
    assert eps.convergedReasonView() == (" Linear eigensolve did not converge due to CONVERGED_ITERATING; "
                                         "iterations 0\n")
    with pytest.raises(sg.SlepcError) as e:
        eps.errorView()
    assert e.value.code == PETSC_ERR_ORDER
    with pytest.raises(sg.SlepcError) as e:
        eps.valuesView()
    assert e.value.code == PETSC_ERR_ORDER
    eps.destroy()


def test_binary_calls_reject_ascii_viewers(lib, tmp_path):
    v = open_ascii(lib, tmp_path / "m.txt")
    A = P()
    assert lib.MatCreate(0, ctypes.byref(A)) == 0
    assert lib.MatLoad(A, v) == PETSC_ERR_SUP
    assert lib.MatDestroy(ctypes.byref(A)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0


# -------------------------------------------------------------------------------------------------------------
# monitors: the built-in printers called directly (host code), against the reference's printed monitor lines
# -------------------------------------------------------------------------------------------------------------
import json  # noqa: E402
import os  # noqa: E402
import re  # noqa: E402

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))
D = ctypes.c_double


def removed(line):
    """test23.c's output filter: error estimates become 'removed'."""
    return re.sub(r"[0-9]\.[0-9]*e-([0-9]*)", "removed", line)


def call_monitor(lib, name, vf, its, nconv, er, ei, es):
    n = len(er)
    f = getattr(lib, name)
    f.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(D),
                  ctypes.c_int, P]
    eps = sg.EPS().create()
    rc = f(eps.handle, its, nconv, (D * n)(*er), (D * n)(*ei), (D * n)(*es), n, vf)
    eps.destroy()
    return rc


def vf_on(lib, path, creator="PetscViewerAndFormatCreate"):
    v = open_ascii(lib, path)
    vf = P()
    getattr(lib, creator).argtypes = [P, ctypes.c_int, ctypes.POINTER(P)] if creator == "PetscViewerAndFormatCreate" \
        else [P, ctypes.c_int, P, ctypes.POINTER(P)]
    if creator == "PetscViewerAndFormatCreate":
        assert lib.PetscViewerAndFormatCreate(v, PETSC_VIEWER_DEFAULT, ctypes.byref(vf)) == 0
    else:
        assert lib.EPSMonitorConvergedCreate(v, PETSC_VIEWER_DEFAULT, None, ctypes.byref(vf)) == 0
    return v, vf


def test_monitor_first_prints_the_reference_lines(lib, tmp_path):
    g = G["test23_2"]
    path = tmp_path / "mon.txt"
    v, vf = vf_on(lib, path)
    er, ei = [20.0 - 1e-9] + [19.0 - 1e-12] + [18.0] * 14, [0.0] * 16
    assert call_monitor(lib, "EPSMonitorFirst", vf, 1, 0, er, ei, [1.2e-4, 3e-5] + [1.0] * 14) == 0
    assert call_monitor(lib, "EPSMonitorFirst", vf, 2, 1, er, ei, [1e-12, 1.7e-8] + [1.0] * 14) == 0
    assert call_monitor(lib, "EPSMonitorFirst", vf, 3, 16, er, ei, [0.0] * 16) == 0  # all converged: no line
    assert lib.PetscViewerAndFormatDestroy(ctypes.byref(vf)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0
    assert [removed(l) for l in path.read_text().splitlines()] == g["monitor"]


def test_monitor_all_and_converged_formats(lib, tmp_path):
    path = tmp_path / "all.txt"
    v, vf = vf_on(lib, path)
    assert call_monitor(lib, "EPSMonitorAll", vf, 3, 1, [6.0, 2.5, -1.25], [0.0, 0.5, -0.5],
                        [0.0, 1e-3, 1e-3]) == 0
    assert lib.PetscViewerAndFormatDestroy(ctypes.byref(vf)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0
    assert path.read_text() == ("  3 EPS nconv=1 Values (Errors) 6. (0.00000000e+00) 2.5+0.5i (1.00000000e-03)"
                                " -1.25-0.5i (1.00000000e-03)\n")
    path = tmp_path / "conv.txt"
    v, vf = vf_on(lib, path, "EPSMonitorConvergedCreate")
    er, ei = [6.0, 5.0, 4.0], [0.0] * 3
    assert call_monitor(lib, "EPSMonitorConverged", vf, 1, 0, er, ei, [1e-3] * 3) == 0
    assert call_monitor(lib, "EPSMonitorConverged", vf, 2, 2, er, ei, [0.0, 0.0, 1e-3]) == 0
    assert call_monitor(lib, "EPSMonitorConverged", vf, 3, 2, er, ei, [0.0, 0.0, 1e-3]) == 0
    assert lib.EPSMonitorConvergedDestroy(ctypes.byref(vf)) == 0
    assert lib.PetscViewerDestroy(ctypes.byref(v)) == 0
    assert path.read_text() == ("  2 EPS converged value (error) #0 6. (0.00000000e+00)\n"
                                "  2 EPS converged value (error) #1 5. (0.00000000e+00)\n")


def test_options_monitors_names_and_views(lib, tmp_path):
    """-eps_monitor*, -eps_view_values, -eps_error_*, -eps_converged_reason parse with viewer specs; draw viewers
    are ignored; an unknown format is an error; PetscObjectSetName is what MATLAB reports print."""
    sg.initialize(["prog", "-eps_monitor", ":" + str(tmp_path / "m.txt"), "-eps_monitor_all", "draw::draw_lg",
                   "-eps_monitor_conv", "-eps_view_values", ":" + str(tmp_path / "v.txt") + ":ascii_matlab",
                   "-eps_error_relative", "::ascii_info_detail", "-eps_converged_reason", "-eps_nev", "3"])
    eps = sg.EPS().create()
    eps.setFromOptions()
    assert eps.getDimensions()[0] == 3
    eps.setName("myeps")
    lib.PetscObjectGetName.argtypes = [P, ctypes.POINTER(ctypes.c_char_p)]
    name = ctypes.c_char_p()
    assert lib.PetscObjectGetName(eps.handle, ctypes.byref(name)) == 0 and name.value == b"myeps"
    eps.monitorCancel()
    eps.destroy()
    sg.initialize(["prog", "-eps_view_values", "::ascii_nonsense"])
    eps = sg.EPS().create()
    with pytest.raises(sg.SlepcError) as e:
        eps.setFromOptions()
    assert e.value.code == PETSC_ERR_SUP
    eps.destroy()
    sg.initialize(["prog"])


def test_eps_view_matches_the_reference_block(lib):
    """EPSView of test23.c's configuration (named "eps", NHEP, largest real, nev 1, ncv = mpd = 6, 100 iterations)
    after EPSSetFromOptions and before EPSSetUp: the EPS Object block of test23_1.out, apart from its balancing and residual-tracking lines
    (options not provided here), the tolerance (the test filters it) and purification (on until EPSSetUp turns it
    off for a standard problem); then the BV, DS and ST objects."""
    A = sg.Mat(*__import__("slepc_gb300.matgen", fromlist=["x"]).laplacian_1d(30))
    eps = sg.EPS().create()
    eps.setOperators(A)
    eps.setProblemType(sg.EPS.ProblemType.NHEP)
    eps.setName("eps")
    eps.setWhichEigenpairs("LR")
    eps.setDimensions(1, 6, 6)
    eps.setTolerances(max_it=100)
    text = eps.view().splitlines()
    # before EPSSetFromOptions (test23.c:43) the ST and DS have no type yet, as in the reference
    assert "  type not yet set" in text and "  type: nhep" not in text
    eps.setFromOptions()
    text = eps.view().splitlines()
    skip = ("balancing", "computing all residuals", "tolerance", "purification")
    ours = [l for l in text[:text.index("BV Object: 1 MPI process")] if not any(k in l for k in skip)]
    ref = [l for l in G["test23_1"]["eps_view"] if not any(k in l for k in skip)]
    assert ours == ref
    assert "DS Object: 1 MPI process" in text and "  type: nhep" in text and "  type: shift" in text
    eps.destroy()


def test_options_prefix_as_test19(lib):
    """test19.c's prefix handling: "check_" + "myprefix_", options -check_myprefix_eps_nev 2 (an unprefixed -eps_nev
    belongs to no-prefix objects); the converged-reason line names the prefix; -check_myprefix_st_type sinvert is
    not provided (the spectral transformation is the shift of 0)."""
    eps = sg.EPS().create()
    eps.setOptionsPrefix("check_")
    eps.appendOptionsPrefix("myprefix_")
    assert eps.getOptionsPrefix() == "check_myprefix_"
    sg.initialize(["test19", "-check_myprefix_eps_nev", "2", "-eps_nev", "7"])
    try:
        eps.setFromOptions()
        assert eps.getDimensions()[0] == 2
        assert eps.convergedReasonView() == ("check_myprefix_ Linear eigensolve did not converge due to "
                                             "CONVERGED_ITERATING; iterations 0\n")
        sg.initialize(["test19", "-check_myprefix_st_type", "sinvert"])
        with pytest.raises(sg.SlepcError) as e:
            eps.setFromOptions()
        assert e.value.code == PETSC_ERR_SUP
        sg.initialize(["test19", "-check_myprefix_st_type", "shift", "-check_myprefix_st_shift", "0"])
        eps.setFromOptions()
    finally:
        sg.initialize(["prog"])
    eps.setOptionsPrefix(None)
    assert eps.getOptionsPrefix() is None
    eps.destroy()


def test_st_object_and_problem_queries(lib):
    """EPSGetST gives the shift-0 transformation: STSetType(shift) and STSetShift(0) are accepted, sinvert and
    nonzero shifts are PETSC_ERR_SUP; EPSIsHermitian/Generalized/Positive follow the problem type."""
    from slepc_gb300 import matgen
    A = sg.Mat(*matgen.laplacian_1d(20))
    B = sg.Mat(*matgen.diagonal(np.ones(20)))
    eps = sg.EPS().create()
    eps.setOperators(A, B)
    st = P()
    lib.EPSGetST.argtypes = [P, ctypes.POINTER(P)]
    assert lib.EPSGetST(eps.handle, ctypes.byref(st)) == 0 and st.value
    for f, a in (("STSetType", [P, ctypes.c_char_p]), ("STSetShift", [P, ctypes.c_double]),
                 ("STGetNumMatrices", [P, ctypes.POINTER(ctypes.c_int)]), ("STGetType", [P, ctypes.POINTER(ctypes.c_char_p)]),
                 ("EPSIsHermitian", [P, ctypes.POINTER(ctypes.c_int)]), ("EPSIsGeneralized", [P, ctypes.POINTER(ctypes.c_int)]),
                 ("EPSIsPositive", [P, ctypes.POINTER(ctypes.c_int)])):
        getattr(lib, f).argtypes = a
    assert lib.STSetType(st, b"shift") == 0 and lib.STSetShift(st, 0.0) == 0
    assert lib.STSetType(st, b"sinvert") == PETSC_ERR_SUP and lib.STSetShift(st, 1.5) == PETSC_ERR_SUP
    t, nm = ctypes.c_char_p(), ctypes.c_int()
    assert lib.STGetType(st, ctypes.byref(t)) == 0 and t.value == b"shift"
    assert lib.STGetNumMatrices(st, ctypes.byref(nm)) == 0 and nm.value == 2
    flags = {}
    for ptype, want in ((sg.EPS.ProblemType.GHEP, (1, 1, 1)), (sg.EPS.ProblemType.GNHEP, (0, 1, 0)),
                        (sg.EPS.ProblemType.HEP, (1, 0, 0)), (sg.EPS.ProblemType.NHEP, (0, 0, 0))):
        eps.setProblemType(ptype)
        got = []
        for f in ("EPSIsHermitian", "EPSIsGeneralized", "EPSIsPositive"):
            b = ctypes.c_int(-1)
            assert getattr(lib, f)(eps.handle, ctypes.byref(b)) == 0
            got.append(b.value)
        flags[ptype] = tuple(got)
        assert tuple(got) == want, (ptype, got)
    eps.destroy()


def test_initial_space_of_several_vectors(lib):
    """EPSSetInitialSpace with several vectors is accepted (the factorisation starts from the first, as in the
    reference); a negative count is an error."""
    eps = sg.EPS().create()
    eps.setInitialSpace([np.ones(20), np.arange(20.0), np.zeros(20)])
    lib.EPSSetInitialSpace.argtypes = [P, ctypes.c_int, P]
    assert lib.EPSSetInitialSpace(eps.handle, -1, None) == 63
    eps.destroy()
