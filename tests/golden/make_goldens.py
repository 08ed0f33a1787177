"""Regenerate reference_outputs.json from the reference's expected-output files (run with SLEPC_REFERENCE set to a SLEPc
source tree; other machines use the committed JSON).  Only the printed eigenvalues/norms of the Krylov-Schur-path tests are
extracted, with the lines EPSErrorView printed; each entry records the file it came from and the options of that
test.  The real matrix those tests read from a PETSc binary file (share/slepc/datafiles/matrices/rdb200.petsc)
is converted to CSR arrays in rdb200.npz by an independent big-endian reader, as are bfw62a/bfw62b (ex7.c)."""
import json
import os
import re

import numpy as np

REF = os.environ.get("SLEPC_REFERENCE", "")
if not REF:
    raise SystemExit("set SLEPC_REFERENCE to the root of the SLEPc 3.22 source tree")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_outputs.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def floats(line):
    return [float(x) for x in re.findall(r"-?\d+\.\d+", line)]


def main():
    g = {}
    # 2-D Laplacian 72x72, -eps_nev 4 -eps_ncv 20 (src/eps/tutorials/ex2.c TEST 1)
    txt = read("src/eps/tutorials/output/ex2_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["ex2_1"] = {"source": "src/eps/tutorials/output/ex2_1.out", "grid": [72, 72], "nev": 4, "ncv": 20,
                  "which": "LM", "eigenvalues": floats(line)}
    # 1-D Laplacian n=30, nev 4: largest, smallest (src/eps/tests/test2.c TEST 1_krylovschur)
    txt = read("src/eps/tests/output/test2_1.out")
    blocks = re.findall(r"- - - (\w+) eigenvalues - - -.*?\n.*?\n(.*?)\n", txt, flags=re.S)
    g["test2_1"] = {"source": "src/eps/tests/output/test2_1.out", "n": 30, "nev": 4,
                    "tol": max(1000 * 2.220446049250313e-16, 1e-9),
                    "largest": floats(blocks[0][1]), "smallest": floats(blocks[1][1]),
                    # EPS_TARGET_MAGNITUDE, target 2.1, EPSSetExtraction(EPS_HARMONIC) for Krylov-Schur
                    "interior": floats(blocks[2][1]), "target": 2.1}
    txt = read("src/eps/tests/output/test2_3.out")
    blocks = re.findall(r"- - - (\w+) eigenvalues - - -.*?\n.*?\n(.*?)\n", txt, flags=re.S)
    g["test2_3"] = {"source": "src/eps/tests/output/test2_3.out", "n": 32, "nev": 4,
                    "largest": floats(blocks[0][1]), "smallest": floats(blocks[1][1])}
    # Brusselator n=50 (100 unknowns), nev 4, largest real (src/eps/tutorials/ex9.c TEST 1)
    txt = read("src/eps/tutorials/output/ex9_1.out")
    line = [l for l in txt.splitlines() if "i," in l or "i" in l and re.search(r"\d\.\d{5}", l)][-1]
    pairs = re.findall(r"(-?\d+\.\d+)([+-]\d+\.\d+)i", line)
    g["ex9_1"] = {"source": "src/eps/tutorials/output/ex9_1.out", "N": 50, "nev": 4, "which": "LR",
                  "eigenvalues": [[float(a), float(b)] for a, b in pairs]}
    # DSHEP compact arrow-tridiagonal n=9, l=2, k=5 (src/sys/classes/ds/tests/test3.c TEST 1)
    txt = read("src/sys/classes/ds/tests/output/test3_1.out")
    vals = txt.split("Computed eigenvalues =")[1].split()
    g["ds_test3_1"] = {"source": "src/sys/classes/ds/tests/output/test3_1.out", "n": 9, "l": 2, "k": 5,
                       "which": "LM", "eigenvalues": [float(v) for v in vals[:9]]}
    # DSNHEP Grcar n=10 (src/sys/classes/ds/tests/test1.c TEST 1)
    txt = read("src/sys/classes/ds/tests/output/test1_1.out")
    body = txt.split("Computed eigenvalues =")[1]
    pairs = re.findall(r"(-?\d+\.\d+)\+-(\d+\.\d+)i", body)
    rn = re.search(r"rnorm for 3rd vector = (\d+\.\d+)", txt)
    nv = re.search(r"Norm of 1st vector = (\d+\.\d+)", txt)
    g["ds_test1_1"] = {"source": "src/sys/classes/ds/tests/output/test1_1.out", "n": 10, "which": "LM",
                       "eigenvalues_abs_imag": [[float(a), float(b)] for a, b in pairs],
                       "rnorm_3rd": float(rn.group(1)), "norm_1st": float(nv.group(1))}
    # rdb200 (200 x 200, non-symmetric), EPS_NHEP defaults, -eps_nev 4 (src/eps/tutorials/ex4.c TEST 1)
    txt = read("src/eps/tutorials/output/ex4_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    its = int(re.search(r"Number of iterations of the method: (\d+)", txt).group(1))
    g["ex4_1"] = {"source": "src/eps/tutorials/output/ex4_1.out", "matrix": "rdb200.npz", "nev": 4, "tol": 1e-8,
                  "which": "LM", "iterations": its, "eigenvalues": floats(line)}
    raw = open(os.path.join(REF, "share/slepc/datafiles/matrices/rdb200.petsc"), "rb").read()
    classid, m, n, nz = np.frombuffer(raw[:16], dtype=">i4")
    assert classid == 1211216 and len(raw) == 16 + 4 * m + 12 * nz
    lens = np.frombuffer(raw[16:16 + 4 * m], dtype=">i4").astype(np.int32)
    cols = np.frombuffer(raw[16 + 4 * m:16 + 4 * m + 4 * nz], dtype=">i4").astype(np.int32)
    vals = np.frombuffer(raw[16 + 4 * m + 4 * nz:], dtype=">f8").astype(np.float64)
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    np.savez(os.path.join(os.path.dirname(OUT), "rdb200.npz"), rowptr=rowptr, colidx=cols, vals=vals,
             shape=np.array([m, n], dtype=np.int32))
    # GHEP: 2-D Laplacian 18x18 with B = diag(2/log(i+2)), nev 4, tol PETSC_SMALL, EPS_CONV_NORM, EPSErrorView with
    # EPS_ERROR_BACKWARD (src/eps/tests/test1.c TEST 1, krylovschur)
    txt = read("src/eps/tests/output/test1_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["test1_1"] = {"source": "src/eps/tests/output/test1_1.out", "grid": [18, 18], "nev": 4, "tol": 1e-10,
                    "conv": "norm", "max_it": 1500, "which": "LM", "eigenvalues": floats(line),
                    "orthogonality": "Level of orthogonality below the tolerance" in txt}
    # -eps_monitor and -eps_view_values ::ascii_matlab on diag(1..20), LR, nev 1 (src/eps/tests/test23.c TEST 2);
    # the test's filter replaced the error estimates with "removed"
    lines = read("src/eps/tests/output/test23_2.out").splitlines()
    g["test23_2"] = {"source": "src/eps/tests/output/test23_2.out", "n": 20, "which": "LR", "nev": 1,
                     "monitor": [l for l in lines if "EPS nconv=" in l],
                     "values_matlab": [l.strip() for l in lines if "Lambda_" in l or l.strip().endswith("e+01")
                                       or l.strip() == "];"]}
    # Markov random walk m=15 (n=120), NHEP, largest real, nev 4, with and without locking (src/eps/tutorials/ex5.c
    # TEST 1; its filter maps 0.90424 -> 0.90423 and 0.85715 -> 0.85714)
    txt = read("src/eps/tutorials/output/ex5_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["ex5_1"] = {"source": "src/eps/tutorials/output/ex5_1.out", "m": 15, "nev": 4, "which": "LR", "tol": 1e-8,
                  "eigenvalues": floats(line), "filter": [["0.90424", "0.90423"], ["0.85715", "0.85714"]]}
    # 1-D Laplacian n=30, HEP, nev 4, largest magnitude, tol 1000 eps (src/eps/tests/test4.c TEST 1, krylovschur)
    txt = read("src/eps/tests/output/test4_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["test4_1"] = {"source": "src/eps/tests/output/test4_1.out", "n": 30, "nev": 4, "which": "LM",
                    "tol": 1000 * 2.220446049250313e-16, "eigenvalues": floats(line)}
    # diag(1..30), HEP, nev 4, largest magnitude, tol PETSC_SMALL (src/eps/tests/test6.c TEST 1, krylovschur)
    txt = read("src/eps/tests/output/test6_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["test6_1"] = {"source": "src/eps/tests/output/test6_1.out", "n": 30, "nev": 4, "which": "LM", "tol": 1e-10,
                    "eigenvalues": floats(line)}
    # graph Laplacian of a 10 x 10 mesh (degree on the diagonal), HEP, smallest real, nev 4, restart 0.2, the
    # constant vector as deflation space (src/eps/tutorials/ex11.c TEST 1)
    txt = read("src/eps/tutorials/output/ex11_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["ex11_1"] = {"source": "src/eps/tutorials/output/ex11_1.out", "grid": [10, 10], "nev": 4, "which": "SR",
                   "keep": 0.2, "tol": 1e-8, "eigenvalues": floats(line)}
    # 1-D Laplacian n=30, HEP, smallest real, nev 4, EPS_CONV_ABS, tol 1e-8, with the exact eigenvectors of the two
    # lowest eigenvalues, sin(pi j (i+1)/(n+1)) sqrt(2/(n+1)), as deflation space (src/eps/tests/test24.c TEST 1, -ncon
    # 2; the test's solver is LOBPCG, the printed eigenvalues are those of the deflated problem)
    txt = read("src/eps/tests/output/test24_1.out")
    line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
    g["test24_1"] = {"source": "src/eps/tests/output/test24_1.out", "n": 30, "ncon": 2, "nev": 4, "which": "SR",
                     "conv": "abs", "tol": 1e-8, "eigenvalues": floats(line)}
    # EPSView of a Krylov-Schur NHEP solve, largest real (src/eps/tests/test23.c TEST 1): the EPS Object block
    lines = read("src/eps/tests/output/test23_1.out").splitlines()
    i0 = next(i for i, l in enumerate(lines) if l.startswith("EPS Object"))
    i1 = next(i for i, l in enumerate(lines) if l.startswith("BV Object"))
    g["test23_1"] = {"source": "src/eps/tests/output/test23_1.out", "eps_view": lines[i0:i1]}
    # 1-D Laplacian n=18, smallest real, nev 1: the default ncv (16), then ncv + 2 = 18 = n, a full basis
    # (src/eps/tests/test20.c TEST 1, krylovschur)
    lines = read("src/eps/tests/output/test20_1.out").splitlines()
    g["test20_1"] = {"source": "src/eps/tests/output/test20_1.out", "n": 18, "nev": 1, "which": "SR",
                     "tol": max(1000 * 2.220446049250313e-16, 1e-9), "ncv": [16, 18],
                     "eigenvalues": [floats(l)[0] for l in lines if re.search(r"\d\.\d{5}", l)]}
    # GNHEP from PETSc binary files bfw62a / bfw62b (62 x 62, B not diagonal), nev 4, largest magnitude, tol 1e-8
    # (src/eps/tutorials/ex7.c TEST 1), and the pencil (A, A) whose eigenvalues are all 1 (TEST 3)
    for key, src in (("ex7_1", "src/eps/tutorials/output/ex7_1.out"), ("ex7_3", "src/eps/tutorials/output/ex7_3.out")):
        txt = read(src)
        line = [l for l in txt.splitlines() if re.search(r"\d\.\d{5}", l)][-1]
        pairs = re.findall(r"(-?\d+\.\d+)(?:([+-]\d+\.\d+)i)?", line)
        g[key] = {"source": src, "matrices": ["bfw62a.npz", "bfw62b.npz" if key == "ex7_1" else "bfw62a.npz"],
                  "nev": 4, "which": "LM", "tol": 1e-8,
                  "iterations": int(re.search(r"Number of iterations of the method: (\d+)", txt).group(1)),
                  "eigenvalues": [[float(a), float(b) if b else 0.0] for a, b in pairs]}
    for name in ("bfw62a", "bfw62b"):
        raw = open(os.path.join(REF, "share/slepc/datafiles/matrices/%s.petsc" % name), "rb").read()
        classid, m, n, nz = np.frombuffer(raw[:16], dtype=">i4")
        assert classid == 1211216 and len(raw) == 16 + 4 * m + 12 * nz
        lens = np.frombuffer(raw[16:16 + 4 * m], dtype=">i4").astype(np.int32)
        cols = np.frombuffer(raw[16 + 4 * m:16 + 4 * m + 4 * nz], dtype=">i4").astype(np.int32)
        vals = np.frombuffer(raw[16 + 4 * m + 4 * nz:], dtype=">f8").astype(np.float64)
        np.savez(os.path.join(os.path.dirname(OUT), name + ".npz"),
                 rowptr=np.concatenate([[0], np.cumsum(lens)]).astype(np.int32), colidx=cols, vals=vals,
                 shape=np.array([m, n], dtype=np.int32))
    # the text EPSErrorView prints (the "All requested ..." line and the eigenvalue line), per solve of each test
    for key in ("ex2_1", "ex9_1", "ex4_1", "test2_1", "test2_3", "test1_1", "ex5_1", "test4_1", "test6_1", "ex7_1",
                "ex7_3", "ex11_1"):
        lines = read(g[key]["source"]).splitlines()
        g[key]["errorview"] = [[lines[i], lines[i + 1]] for i, l in enumerate(lines)
                               if l.startswith(" All requested eigenvalues")]
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
