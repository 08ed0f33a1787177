"""CPU model of the integer-pipe Gram-Schmidt pair (slepc_gb300/csrc/k_gs_ix.cu with the helpers of gs_fixed.cuh):
the 54-bit fixed-point split, the exact 64-bit partial sums and their bounds, the 128-bit combine, the accumulator
with a binary exponent, the once-rounded conversion to a double, the row partition of the dot half and the tile
bookkeeping of the update half.  The constants and formulas are the kernels'; a change there must be mirrored here.
Every integer is a Python int, checked against the two's complement range the kernel stores it in."""
import math
import random
from fractions import Fraction

import numpy as np
import pytest

IX_THREADS, IX_GROUP, IX_GMAX, IX_MAXJ = 512, 512, 4, 144
IX_TMAX = IX_GROUP * IX_GMAX
IU_THREADS = 256
IU_ROWS = 2 * IU_THREADS
INT_MIN = None  # the empty accumulator


def i64(x):
    assert -(1 << 63) <= x < (1 << 63), x
    return x


def expo(v):
    """gt_expo: the biased exponent field"""
    return (np.float64(v).view(np.uint64) >> np.uint64(52)).item() & 0x7FF


def escale(E):
    """gt_escale"""
    if E == 0:
        return -128
    return max(-127, min(127, E - 1022))


def split53(v, e):
    """ix_split53: (H, L, ok) with X = trunc(v 2^(53-e)) = H 2^26 + L"""
    u = np.float64(v).view(np.uint64).item()
    E = (u >> 52) & 0x7FF
    s0 = 1022 + e - E
    m = (u & ((1 << 52) - 1)) | (1 << 52)
    sh = s0 if 0 <= s0 <= 63 else 63
    x = m >> sh
    sgn = -1 if (u >> 63) else 1
    H, L = sgn * (x >> 26), sgn * (x & ((1 << 26) - 1))  # the sign of v on both halves
    assert abs(H) < (1 << 27) and abs(L) < (1 << 26)
    return H, L, s0 >= 0


def mac(acc, Hv, Lv, Hx, Lx):
    hh, mm, ll = acc
    hh = i64(hh + Hv * Hx)
    mm = i64(mm + Hv * Lx + Lv * Hx)
    ll = i64(ll + Lv * Lx)
    return hh, mm, ll


def combine(hh, mm, ll):
    """ix_combine: the exact value as a 128-bit two's complement integer"""
    P = (hh << 52) + (mm << 26) + ll
    assert -(1 << 127) <= P < (1 << 127)
    return P


def acc_add(A, P, kp):
    """ix_acc_add on (value, k): A = None when empty"""
    if P == 0:
        return A
    if A is None:
        V, k = P, kp
    else:
        V, k = A
        if kp > k:
            V >>= min(kp - k, 127)
            k = kp
        elif kp < k:
            P >>= min(k - kp, 127)
        V += P
    assert -(1 << 127) <= V < (1 << 127)
    if (V >> 123) not in (0, -1):  # (hi >> 59) != (hi >> 63)
        V >>= 4
        k += 4
    return V, k


def to_double(P, k):
    """ix_to_double: P 2^k rounded once to nearest even"""
    if P == 0:
        return 0.0
    return float(Fraction(P) * Fraction(2) ** k)


def to_double_bits(P, k):
    """the kernel's bit construction, step by step"""
    neg = P < 0
    mag = -P if neg else P
    if mag == 0:
        return 0.0
    h, lo = mag >> 64, mag & ((1 << 64) - 1)
    sh = 0
    if h == 0:
        h, lo, sh = lo, 0, 64
    lz = 64 - h.bit_length()
    if lz > 0:
        h = ((h << lz) | (lo >> (64 - lz))) & ((1 << 64) - 1)
        lo = (lo << lz) & ((1 << 64) - 1)
    sh += lz
    m = h >> 11
    rest = h & 0x7FF
    if (rest & 0x400) and ((rest & 0x3FF) or lo or (m & 1)):
        m += 1
    e2 = k - sh + 75
    if m >> 53:
        m >>= 1
        e2 += 1
    be = e2 + 1075
    if be < 1 or be > 2046:
        return math.ldexp(-float(m) if neg else float(m), e2)
    bits = (int(neg) << 63) | (be << 52) | (m & ((1 << 52) - 1))
    return np.uint64(bits).view(np.float64).item()


def test_split_is_the_truncated_fixed_point():
    rng = random.Random(1)
    for _ in range(4000):
        e = rng.randint(-40, 5)
        v = rng.uniform(-1, 1) * 2.0 ** (e - rng.choice([0, 0, 1, 3, 20, 60]))
        H, L, ok = split53(v, e)
        assert ok
        X = H * (1 << 26) + L
        exact = Fraction(v) * Fraction(2) ** (53 - e)
        assert X == int(exact)  # truncation toward zero
        assert abs(X) < (1 << 53) and abs(H) < (1 << 27) and abs(L) < (1 << 26)
        # the top binade keeps the whole significand
        if abs(v) >= 2.0 ** (e - 1):
            assert Fraction(X) == exact
    # a value at or above its scale, and a non-finite one, are flagged
    assert not split53(1.0, 0)[2] and not split53(-3.0, 1)[2] and not split53(float("inf"), 127)[2]
    assert split53(0.999, 0)[2] and split53(0.0, -128)[2] and split53(-0.0, 5)[2]
    assert split53(0.0, -128)[:2] == (0, 0) and split53(5e-324, 0)[:2] == (0, 0)


def test_partial_sums_fit_their_registers_at_the_longest_runs():
    # half A: a lane sums 16 G <= 64 rows of a column per tile, then 32 lanes meet in 128 bits;
    # half B: a row sums J <= 144 columns.  Every term at its extreme magnitude (twice: two products per step).
    runs = max(16 * IX_GMAX, IX_MAXJ)
    assert runs == 144
    Hmax, Lmax = (1 << 27) - 1, (1 << 26) - 1
    for sh in (1, -1):
        acc = (0, 0, 0)
        for _ in range(runs):
            acc = mac(acc, sh * Hmax, Lmax, -Hmax, Lmax)
            acc = mac(acc, -sh * Hmax, Lmax, -Hmax, Lmax)
        combine(*acc)
    # 128-bit combine of a run, then a few thousand chunk folds at the top scale stay in range
    P = combine(runs * Hmax * Hmax, 2 * runs * Hmax * Lmax, runs * Lmax * Lmax)
    assert combine(-runs * Hmax * Hmax, -2 * runs * Hmax * Lmax, -runs * Lmax * Lmax) == -P
    assert abs(32 * P) < (1 << 127)  # the lanes' butterfly
    A = None
    for _ in range(5000):
        A = acc_add(A, P, -106)
    assert A[1] >= -106


def test_dot_model_is_exact_before_one_rounding():
    rng = np.random.default_rng(7)
    for n in (1, 5, 300, 2049):
        v = rng.standard_normal(n)
        v /= np.linalg.norm(v)
        u = rng.standard_normal(n) * 3.7
        ev = escale(max(expo(x) for x in v))
        eu = escale(max(expo(x) for x in u))
        acc = (0, 0, 0)
        for a, b in zip(v, u):
            Hv, Lv, okv = split53(a, ev)
            Hu, Lu, oku = split53(b, eu)
            assert okv and oku
            acc = mac(acc, Hv, Lv, Hu, Lu)
        P = combine(*acc)
        exact_fixed = sum(int(Fraction(a) * Fraction(2) ** (53 - ev)) * int(Fraction(b) * Fraction(2) ** (53 - eu))
                          for a, b in zip(v, u))
        assert P == exact_fixed
        got = to_double(P, ev + eu - 106)
        exact = sum(Fraction(a) * Fraction(b) for a, b in zip(v, u))
        # truncation of the inputs: at most 2^(e-53) per value
        bound = Fraction(2) ** (ev - 53) * sum(abs(Fraction(b)) for b in u) + \
            Fraction(2) ** (eu - 53) * sum(abs(Fraction(a)) for a in v) + abs(exact) * Fraction(2) ** -52
        assert abs(Fraction(got) - exact) <= bound
        assert abs(got - float(exact)) <= 4e-16 * np.linalg.norm(u) * max(1.0, math.sqrt(n) / 8)


def test_conversion_rounds_once_to_nearest_even():
    rng = random.Random(3)
    cases = [1, -1, (1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6, -(1 << 127), (1 << 127) - 1, 3 << 70]
    cases += [rng.randrange(-(1 << 127), 1 << 127) >> rng.randrange(0, 120) for _ in range(3000)]
    for P in cases:
        for k in (-230, -106, 0, 40):
            want = to_double(P, k)
            assert to_double_bits(P, k) == want, (P, k)


def test_accumulator_drops_only_bits_far_below_its_scale():
    rng = random.Random(11)
    for _ in range(200):
        A = None
        total = Fraction(0)
        top = None
        for _ in range(rng.randint(1, 40)):
            P = rng.randrange(-(1 << 113), 1 << 113)
            kp = rng.randint(-140, -90)
            A = acc_add(A, P, kp)
            total += Fraction(P) * Fraction(2) ** kp
            top = kp if top is None else max(top, kp)
        V, k = A
        err = abs(Fraction(V) * Fraction(2) ** k - total)
        assert err <= 60 * Fraction(2) ** (k)  # a few units of the accumulator's last place per fold
        assert k <= top + 8


def groups_per_tile(n, sms=152):
    """gs_ix_groups: the largest G in 4..1 whose tiles spread over the grid within 2% of an even split"""
    best, best_w = 1, 1e30
    for G in range(IX_GMAX, 0, -1):
        nt = -(-n // (IX_GROUP * G))
        gr = min(nt, sms)
        w = (-(-nt // gr) * gr) / nt
        if w <= 1.02:
            return G
        if w < best_w:
            best, best_w = G, w
    return best


def test_tile_choice_balances_the_grid():
    assert groups_per_tile(128 ** 3) == 3            # 1366 tiles of 1536 rows: 9 waves of 152 blocks
    assert groups_per_tile(64 ** 3) in (1, 2, 4)
    assert groups_per_tile(1) == 4 and groups_per_tile(10 ** 6) >= 1


@pytest.mark.parametrize("n", [1, 3, 511, 512, 513, 2047, 5000, 13824])
@pytest.mark.parametrize("J", [1, 2, 17, 75, 143, 144])
def test_dot_half_partition_covers_every_row_once(n, J):
    """k_gs_dot_ix: tiles of 512 G rows round-robin over the grid; warp w takes columns w + 16 kk; lane l of a load
    group gq takes rows 512 gq + 2 l + 64 i and the next one (i < 8)"""
    G = groups_per_tile(n)
    TR = IX_GROUP * G
    ntile = -(-n // TR)
    ntiles128 = -(-n // 128)
    grid = min(152, ntile)
    seen = np.zeros((J, n), dtype=np.int64)
    for blk in range(grid):
        for t in range(blk, ntile, grid):
            t128 = (t * TR) >> 7
            nt128 = min(TR >> 7, ntiles128 - t128)
            assert 1 <= nt128 <= 32 and t128 + nt128 <= ntiles128   # the lanes reading the exponent table
            for warp in range(IX_THREADS // 32):
                nk = (J - warp + 15) // 16 if warp < J else 0
                for kk in range(nk):
                    c = warp + 16 * kk
                    assert c < J
                    for gq in range(G):
                        for lane in range(32):
                            for i in range(8):
                                rr = IX_GROUP * gq + 2 * lane + 64 * i  # row in the tile: the split pairs su[rr], su[rr+1]
                                assert rr + 1 < TR <= IX_TMAX
                                for e in (0, 1):
                                    r = t * TR + rr + e
                                    if r < n:
                                        seen[c, r] += 1
    assert (seen == 1).all()
    # a lane sums 16 G <= 64 rows of a column per tile; the raw copies cover the tile in 16-byte row pairs
    assert 16 * G <= 64 and (TR // 2) <= 2 * IX_THREADS


@pytest.mark.parametrize("n", [1, 2, 255, 256, 511, 512, 513, 1000, 4097])
def test_update_half_tiles_and_rows(n):
    """k_gs_update_ix: thread = rows 2 tid, 2 tid + 1 of a 512-row pass; warp w's rows lie in tile 4p + w // 2"""
    npass = -(-n // IU_ROWS)
    ntiles = -(-n // 128)
    ldt = (ntiles + 7) // 8 * 8
    covered = np.zeros(n, dtype=np.int64)
    written = set()
    for p in range(npass):
        for tid in range(IU_THREADS):
            warp = tid // 32
            r = p * IU_ROWS + 2 * tid
            T = (p * IU_ROWS + 64 * warp) >> 7
            for rr in (r, r + 1):
                if rr < n:
                    covered[rr] += 1
                    assert rr // 128 == T < ntiles <= ldt
        for t in range(IU_ROWS // 128):
            Tt = p * (IU_ROWS // 128) + t
            if Tt < ntiles:
                written.add(Tt)
    assert (covered == 1).all()
    assert written == set(range(ntiles))
