"""The reference's own EPS programs compile and link unchanged against include/ and libslepc_gb300.so.

Where the reference tree is given (environment variable SLEPC_REFERENCE, the root of a SLEPc 3.22 source tree; the
tests skip when it is unset), each program is compiled in place from its source with gcc -Wall -Werror and linked against the library; nothing is copied.  Run
without a GPU, a program builds its matrices and options and then stops at EPSSolve with PETSC_ERR_GPU (97) and the
CUDA error: there is no CPU fallback.  With a GPU it solves."""
import os
import shutil
import subprocess

import pytest

import slepc_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SLEPC_REFERENCE", "")
PROGRAMS = ["tutorials/ex1", "tutorials/ex2", "tutorials/ex4", "tutorials/ex5", "tutorials/ex7", "tutorials/ex11",
            "tutorials/ex13", "tutorials/ex44", "tests/test1", "tests/test2", "tests/test3", "tests/test4",
            "tests/test6", "tests/test10", "tests/test14", "tests/test18", "tests/test19", "tests/test20",
            "tests/test23", "tests/test26", "tests/test27", "tests/test28", "tests/test39", "tests/test42"]
# these build their problem and reach EPSSolve on a machine without a GPU (PETSC_ERR_GPU there)
RUN_TO_SOLVE = ["tutorials/ex1", "tutorials/ex13", "tutorials/ex44", "tests/test27", "tests/test28", "tests/test3",
                "tests/test42"]

pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "src", "eps")) or not shutil.which("gcc"),
                                reason="SLEPC_REFERENCE (a SLEPc source tree) is unset, or gcc is missing")


@pytest.fixture(scope="module")
def libdir():
    sg.build()
    return os.path.dirname(sg.LIB_PATH)


@pytest.mark.parametrize("prog", PROGRAMS)
def test_program_compiles_and_links(prog, libdir, tmp_path):
    src = os.path.join(REF, "src", "eps", prog + ".c")
    exe = tmp_path / os.path.basename(prog)
    r = subprocess.run(["gcc", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
                        "-L", libdir, "-lslepc_gb300", "-lm", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]


def test_program_runs_to_the_solve(libdir, tmp_path):
    """ex2 -n 10: the header line, then EPSSolve -- on a machine without a GPU it reports PETSC_ERR_GPU."""
    exe = tmp_path / "ex2"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), os.path.join(REF, "src/eps/tutorials/ex2.c"), "-o",
                    str(exe), "-L", libdir, "-lslepc_gb300", "-lm", "-Wl,-rpath," + libdir], check=True, timeout=120)
    r = subprocess.run([str(exe), "-n", "10", "-eps_nev", "4", "-terse"], capture_output=True, text=True, timeout=600)
    assert "2-D Laplacian Eigenproblem, N=100 (10x10 grid)" in r.stdout
    if r.returncode == 97:
        assert "PETSC ERROR" in r.stderr and "CUDA error" in r.stderr
    else:
        assert r.returncode == 0 and "All requested eigenvalues computed up to the required tolerance" in r.stdout


def test_interface_queries_print_as_the_reference(libdir, tmp_path):
    """test14 (src/eps/tests/test14.c) sets and queries every EPS setting, views the operator, the ST and the DS
    before the solve: everything it prints up to EPSSolve matches the reference's output file line for line."""
    exe = tmp_path / "test14"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), os.path.join(REF, "src/eps/tests/test14.c"), "-o",
                    str(exe), "-L", libdir, "-lslepc_gb300", "-lm", "-Wl,-rpath," + libdir], check=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    with open(os.path.join(REF, "src/eps/tests/output/test14_1.out")) as f:
        expected = f.read()
    before_solve = expected[:expected.index(" Finished")]
    if r.returncode == 97:
        assert r.stdout == before_solve and "CUDA error" in r.stderr
    else:
        assert r.returncode == 0 and r.stdout == expected


@pytest.mark.parametrize("prog", RUN_TO_SOLVE)
def test_program_reaches_the_solve(prog, libdir, tmp_path):
    """Every call before EPSSolve succeeds; the solve itself needs the GPU (PETSC_ERR_GPU without one)."""
    exe = tmp_path / os.path.basename(prog)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), os.path.join(REF, "src", "eps", prog + ".c"), "-o",
                    str(exe), "-L", libdir, "-lslepc_gb300", "-lm", "-Wl,-rpath," + libdir], check=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    if r.returncode == 97:
        assert "EPSSolve(eps) returned 97" in r.stderr and "CUDA error" in r.stderr, r.stderr[-2000:]
    else:
        assert r.returncode == 0, r.stderr[-2000:]
