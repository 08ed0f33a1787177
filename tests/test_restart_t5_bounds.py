"""CPU model of the tcgen05 restart kernel's addressing (k_restart_t5w in slepc_gb300/csrc/k_restart_tc.cu, the
warp-specialised form): for a sweep of problem sizes and restart shapes, every shared-memory, tensor-memory,
scratch, Q-slice and basis access the kernel makes stays inside its allocation, every bulk copy is 16-byte aligned
with a size that is a multiple of 16, the mbarrier transaction and arrival counts stay below their limits, and the
two warp groups' hand-offs pair up.  The constants and formulas are the kernel's; a change there must be mirrored
here."""
import itertools

import pytest

# kernel constants
OZ_SA, OZ_S, OZ_QMAX, OZ_L, OZ_NC = 8, 7, 8, 8, 32
T5_M, T5_NC, T5_KC, T5_THREADS = 128, 64, 32, 512
T5_ASL = T5_M * T5_KC * 2
T5_BSL = T5_NC * T5_KC * 2
T5_STAGE = OZ_SA * T5_ASL + OZ_QMAX * T5_BSL
T5W_TENSOR = 256
T5W_SLICERS = T5_THREADS - T5W_TENSOR
T5W_H = T5W_SLICERS // T5_M
T5_SMEM = 2 * T5_STAGE + (2 + T5W_H) * T5_M * 4 + 9 * 8 + 16 + T5_NC * 4
TMEM_COLS = OZ_L * T5_NC
NUM_SMS = 152
BF16 = 2


def rup(x, m):
    return (x + m - 1) // m * m


def scratch_layout(ld):
    """restart_tc_scratch_bytes / t5_qbytes / t5_abytes / restart_t5_scratch_bytes"""
    kp_max, np_ = rup(ld, 16), rup(ld, OZ_NC)
    tc = OZ_QMAX * np_ * kp_max * BF16 + np_ * 4 + 256
    q = rup(tc, 256)
    a = NUM_SMS * 2 * OZ_SA * rup(ld, 16) * 128 * BF16  # two slice buffers per CTA
    return {"np": np_, "tc": tc, "q": q, "a": a, "total": q + a + 256}


def check(n, ld, K, N, f64=False):
    """f64: the FP64-storage kernel (Q in 8 slices when K <= 128, else 7); otherwise pair storage (7 slices)."""
    assert 0 < K <= ld and 0 < N <= ld and ld <= 144
    lay = scratch_layout(ld)
    np_ = lay["np"]
    kp, ldp = rup(K, 16), rup(ld, 16)
    QS = OZ_QMAX if (f64 and kp <= 128) else OZ_S
    assert kp <= ldp and np_ >= rup(N, 16)            # the launch's own checks
    assert min(QS, OZ_L) * 127 * 128 * kp < (1 << 24)  # every level sum exact in FP32
    assert T5_SMEM <= 227 * 1024
    # shared layout: stages, erow[2][128] + etmp[H][128], nine mbarriers (8-byte aligned), the TMEM slot
    erow = 2 * T5_STAGE
    etmp = erow + 2 * T5_M * 4
    bars = etmp + T5W_H * T5_M * 4
    assert bars % 8 == 0 and bars + 9 * 8 + 4 <= T5_SMEM
    cmax = bars + 9 * 8 + 16                           # per-column exponent maxima (FP64 storage), 64 ints
    assert cmax % 4 == 0 and cmax + T5_NC * 4 <= T5_SMEM
    # the exponent pass: slicing thread st covers row st % 128 with part st // 128 of the columns
    assert T5W_SLICERS % T5_M == 0 and T5W_H >= 1 and T5W_SLICERS < (1 << 20)  # ready[] arrival count
    nk8 = kp // 8
    ntiles = -(-n // T5_M)
    blocks = min(NUM_SMS, ntiles)
    ldv = rup(n, 64)
    v_elems = ldv * (ld + 1)                           # float2 entries of the basis
    # Q slices (cm layout) written by k_oz_qslice: element (t, c, k)
    q_max = ((QS - 1) * nk8 + (kp - 1) // 8) * (np_ // 8) * 64 + ((np_ - 1) // 8) * 64 + 7 * 8 + 7
    assert (q_max + 1) * BF16 <= OZ_QMAX * np_ * kp * BF16
    assert OZ_QMAX * np_ * kp * BF16 + np_ * 4 <= lay["tc"]  # the slices, then the column exponents
    # per-CTA slice scratch: two buffers of OZ_SA x nk8 x 16 x 64 bf16
    per_buf = OZ_SA * nk8 * 16 * 64 * BF16
    per_cta = 2 * per_buf
    assert blocks * per_cta <= lay["a"]
    assert lay["q"] % 16 == 0 and per_buf % 16 == 0
    for tile in range(ntiles):
        r0 = tile * T5_M
        rows = min(T5_M, n - r0)
        # slicing threads read V(r0 + m, a0 + k) for m < rows, k < K; a0 + K <= ld
        for a0 in (0, ld - K):
            last = r0 + rows - 1 + (a0 + K - 1) * ldv
            assert last < v_elems
        # slicing stores: item (m, k8) -> ((s nk8 + k8) 16 + m / 8) 64 + (m % 8) 8, 16 bytes, in buffer j % 2
        top = ((OZ_SA - 1) * nk8 + nk8 - 1) * 16 * 64 + 15 * 64 + 7 * 8 + 8
        assert top * BF16 <= per_buf
    # chunks and stages
    nkc = -(-kp // T5_KC)
    for c0 in range(0, N, T5_NC):
        nch = min(T5_NC, rup(N - c0, 16))
        assert nch % 16 == 0 and 16 <= nch <= 256       # MMA N for M = 128
        assert (OZ_L - 1) * T5_NC + nch <= TMEM_COLS    # level accumulators
        for i in range(nkc):
            kc8 = i * (T5_KC // 8)
            sk8 = min(T5_KC // 8, nk8 - kc8)
            assert sk8 in (2, 4)
            abytes = sk8 * 16 * 128
            bbytes = (nch // 8) * 128
            assert abytes % 16 == 0 and bbytes % 16 == 0
            assert OZ_SA * abytes + QS * sk8 * bbytes < (1 << 20)
            # A copies: source inside the tile's slice buffer, destination inside its slice of the stage
            for sl in range(OZ_SA):
                src_end = ((sl * nk8 + kc8) * 16 * 64) * BF16 + abytes
                assert src_end <= per_buf and abytes <= T5_ASL
                assert per_buf % 16 == 0  # buffer 1 starts 16-byte aligned
            # B copies: source inside the Q slices, destination inside the slice of the stage
            for t, k8 in itertools.product(range(QS), range(sk8)):
                src = (((t * nk8 + kc8 + k8) * (np_ // 8) + c0 // 8) * 64) * BF16
                assert src % 16 == 0 and src + bbytes <= QS * np_ * kp * BF16
                assert k8 * (T5_NC // 8) * 128 + bbytes <= T5_BSL
                assert OZ_SA * T5_ASL + t * T5_BSL + T5_BSL <= T5_STAGE
            # what the tensor cores read per MMA (K-major, no swizzle: 8-row groups at SBO, K core matrices at LBO)
            for j in range(sk8 // 2):
                a_lo = j * 2 * 16 * 128
                a_hi = a_lo + 15 * 128 + 1 * (16 * 128) + 128
                b_lo = j * 2 * (T5_NC // 8) * 128
                b_hi = b_lo + (nch // 8 - 1) * 128 + 1 * (T5_NC // 8) * 128 + 128
                assert a_hi <= T5_ASL and b_hi <= T5_BSL
                assert (2 * T5_STAGE) >> 4 < (1 << 14)  # descriptor start-address field
        # epilogue: tensor warp w reads lanes 32 (w % 4) .. +31 and columns L 64 + col .. +15 for
        # col = 16 (w / 4), + 16 (T5W_TENSOR / 128), .. < nch; every column group is read by one warp per lane quarter
        seen = set()
        for w in range(T5W_TENSOR // 32):
            for col in range(16 * (w // 4), nch, 16 * (T5W_TENSOR // 128)):
                assert 32 * (w % 4) + 31 < 128 and (OZ_L - 1) * T5_NC + col + 16 <= TMEM_COLS
                assert c0 + col < rup(N, 16) <= np_     # fcol entries read are written by k_oz_qslice
                assert (w % 4, col) not in seen
                seen.add((w % 4, col))
        assert seen == {(q, col) for q in range(4) for col in range(0, nch, 16)}
        assert nch <= T5W_TENSOR                        # the column-exponent threads (tid < nch) are tensor threads


@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 1000, 4095, 12167, 27000])
@pytest.mark.parametrize("ld,K,N", [(24, 24, 17), (41, 40, 30), (111, 110, 70), (129, 128, 64), (129, 128, 96),
                                    (129, 75, 128), (144, 143, 143), (144, 16, 16), (33, 1, 1)])
@pytest.mark.parametrize("f64", [False, True])
def test_t5_addressing_in_bounds(n, ld, K, N, f64):
    check(n, ld, K, N, f64)


def test_t5_shared_memory_and_registers_fit():
    # 512 threads x at most 128 registers (ptxas -v: 120 for pair storage, 126 for FP64) fit the SM's 65,536
    # registers; one CTA per SM by TMEM and shared memory
    assert T5_THREADS * 128 <= 65536
    assert 2 * T5_SMEM > 228 * 1024


def test_t5w_handoff_phases():
    """The parities of the two groups' waits pair up: the tensor warps wait ready[j % 2] with parity (j // 2) % 2,
    the phase the slicing warps complete with their (j // 2)-th arrival on that buffer; the slicing warps wait
    done[j % 2] with parity ((j - 2) // 2) % 2 before refilling it, the phase of tile j - 2's write-back."""
    for ntiles_cta in range(1, 12):
        completions = {0: 0, 1: 0}  # per buffer: phases of ready completed so far
        dones = {0: 0, 1: 0}
        for j in range(ntiles_cta):
            b = j % 2
            if j >= 2:
                assert dones[b] >= 1 and ((dones[b] - 1) % 2) == ((j - 2) // 2) % 2
            completions[b] += 1  # the slicing warps' arrivals complete phase completions[b] - 1
            assert (completions[b] - 1) % 2 == (j // 2) % 2
            dones[b] += 1
