"""The C-ABI library builds here (cross-compiled for sm_103a), loads without a GPU and exports every function
declared in include/*.h."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:PetscErrorCode|const char \*)\s+(\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_entry_points():
    names = declared_functions()
    for required in ["EPSCreate", "EPSSetOperators", "EPSSetProblemType", "EPSSetType", "EPSSetDimensions",
                     "EPSSetTolerances", "EPSSetWhichEigenpairs", "EPSSetInitialSpace", "EPSSolve",
                     "EPSGetConverged", "EPSGetEigenpair", "EPSGetIterationNumber", "EPSGetConvergedReason",
                     "EPSComputeError", "EPSDestroy", "EPSKrylovSchurSetRestart", "EPSKrylovSchurSetLocking",
                     "MatMult", "BVDotVec", "BVMultVec", "BVMultInPlace", "BVNorm", "BVNormColumn",
                     "BVOrthonormalizeColumn", "BVMatArnoldi", "BVMatLanczos", "DSSolve", "DSSort", "DSTruncate",
                     "DSVectors", "DSUpdateExtraRow", "MatCreateSeqAIJWithArrays"]:
        assert required in names, required


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_oracle_in_product():
    # the product sources never reference the oracle
    for f in glob.glob(os.path.join(ROOT, "slepc_gb300", "**", "*.*"), recursive=True):
        if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            txt = open(f).read()
            assert "ks_oracle" not in txt and "import oracle" not in txt, f
