"""CPU: the integer-only rounding of the tcgen05 restart's FP64 epilogue (slepc_gb300/csrc/oz_round.h), compiled
for the host, against exact rational arithmetic: X 2^sc with X = H 2^42 + R rounded to nearest (ties to even) for
random, boundary and tie cases, and the integer value of integer-valued floats below 2^24."""
import os
import random
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("ozr") / "oz_round_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", out, os.path.join(HERE, "native", "oz_round_check.cpp")],
                   check=True)
    return out


def run(exe, lines):
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return r.stdout.split("\n")


def expected(H, R, sc):
    X = H * (1 << 42) + R
    v = Fraction(X) * (Fraction(2) ** sc)
    try:
        f = float(v)  # correctly rounded, ties to even
    except OverflowError:
        return None
    # normal range only (the kernel computes anything else in FP64), including a nonzero X that underflows to 0
    if (f != 0.0 or X != 0) and not (2.0 ** -1022 <= abs(f) <= 1.7976931348623157e308):
        return None
    return f


def test_round_x_matches_exact_rounding(exe):
    rng = random.Random(11)
    cases = []
    for _ in range(4000):
        H = rng.randint(-(1 << 33) + 1, (1 << 33) - 1) if rng.random() < 0.8 else rng.randint(-5, 5)
        R = rng.randint(-(1 << 61) + 1, (1 << 61) - 1) >> rng.randint(0, 60)
        sc = rng.randint(-200, 60)
        cases.append((H, R, sc))
    # ties and carries: X with exactly one bit below the 53 kept, odd and even significands, and all-ones
    for p in range(53, 76):
        for m in ((1 << 52) | 1, (1 << 52) | 2, (1 << 53) - 1):
            sh = p - 52
            for low in (1 << (sh - 1), (1 << (sh - 1)) - 1, (1 << (sh - 1)) + 1):
                X = (m << sh) | low
                H, R = X >> 42, X & ((1 << 42) - 1)
                cases += [(H, R, -70), (-H, -R, -70)]
    cases += [(0, 0, 5), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0), (0, (1 << 61) - 1, -60), (0, 5, -1080),
              (1 << 32, 0, 900)]
    out = run(exe, [f"x {H} {R} {sc}" for H, R, sc in cases])
    checked = 0
    for (H, R, sc), line in zip(cases, out):
        ok, bits = line.split()
        want = expected(H, R, sc)
        if want is None:
            assert ok == "0", (H, R, sc)
            continue
        assert ok == "1", (H, R, sc)
        got = struct.unpack("<d", bytes.fromhex(bits)[::-1])[0]
        assert got == want and (got != 0.0 or bits == "0000000000000000"), (H, R, sc, got, want)
        checked += 1
    assert checked > 4000


def test_f2i_exact(exe):
    rng = random.Random(5)
    vals = [0, 1, -1, 2, 3, (1 << 24) - 1, -(1 << 24) + 1, 1 << 23, -(1 << 23)] + \
           [rng.randint(-(1 << 24) + 1, (1 << 24) - 1) for _ in range(2000)]
    lines = [f"f {struct.unpack('<I', struct.pack('<f', float(v)))[0]:x}" for v in vals]
    lines.append(f"f {0x80000000:x}")  # -0.0
    out = run(exe, lines)
    for v, line in zip(vals + [0], out):
        assert int(line) == v
