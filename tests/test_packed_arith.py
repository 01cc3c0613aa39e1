"""Host models of the packed-integer identities the DP kernels rely on
(gotoh.cu), checked exhaustively or on dense random samples:

* the 16x2 row-maximum keep mask: old + 0x8000 - new per half never carries
  or borrows across halves for values in [0, 32766], and its bit 15 is set
  exactly when old >= new (PRMT 0xBB99 spreads that bit over the half);
* the opened-gap flags: with kE = 0 or 1 and kF = 0 or 2 (mod 4),
  (kE | kF) & 3 equals (kE - E4) + (kF - F4), E4 = kE & ~3, F4 = kF & ~3;
* the LOP3 immediate 0xA8 is (a | b) & c;
* the zero-half filter of the strip bookkeeping: (x - 0x10001) & ~x has bit
  15 of a half set whenever that half is zero (no false negatives; it may
  also flag the half above a zero one).
"""
import random

M16 = 0xFFFF
M32 = 0xFFFFFFFF


def prmt_sign_halves(t):
    """PRMT(t, 0, 0xBB99): each half filled with its bit 15."""
    lo = M16 if t & 0x8000 else 0
    hi = M16 if t & 0x80000000 else 0
    return lo | (hi << 16)


def test_row_max_keep_mask():
    rng = random.Random(1)
    edge = [0, 1, 2, 3, 32765, 32766]
    vals = edge + [rng.randrange(0, 32767) for _ in range(300)]
    for oa in vals[:60]:
        for na in vals[:60]:
            ob, nb = rng.choice(vals), rng.choice(vals)
            old = oa | (ob << 16)
            new = na | (nb << 16)
            t = (old + 0x80008000 - new) & M32
            # per half, no carry or borrow crossed: the low half alone gives
            # the same low 16 bits, and the high half is exact too
            assert t & M16 == (oa + 0x8000 - na) & M16
            assert t >> 16 == (ob + 0x8000 - nb) & M16
            keep = prmt_sign_halves(t)
            assert (keep & M16 == M16) == (oa >= na)
            assert (keep >> 16 == M16) == (ob >= nb)
            rmax = (old & keep) | (new & ~keep & M32)
            assert rmax & M16 == max(oa, na) and rmax >> 16 == max(ob, nb)


def test_opened_flags_by_one_lop3():
    for e4 in range(-64, 64, 4):
        for f4 in range(-64, 64, 4):
            for ke_low in (0, 1):
                for kf_low in (0, 2):
                    kE, kF = (e4 + ke_low) & M32, (f4 + kf_low) & M32
                    E4, F4 = kE & ~3 & M32, kF & ~3 & M32
                    adds = ((kE - E4) + (kF - F4)) & M32
                    assert (kE | kF) & 3 == adds


def test_lop3_immediate_a8_is_or_then_and():
    a, b, c = 0xF0, 0xCC, 0xAA  # the LOP3 truth-table convention
    assert (a | b) & c == 0xA8


def test_zero_half_filter_has_no_false_negatives():
    rng = random.Random(2)
    samples = [0, 1, 0x10000, 0x10001, 0xFFFF, 0xFFFF0000, M32, 0x8000, 0x80000000]
    samples += [rng.getrandbits(32) for _ in range(20000)]
    samples += [rng.getrandbits(16) << 16 for _ in range(2000)]  # low half zero
    samples += [rng.getrandbits(16) for _ in range(2000)]        # high half zero
    for x in samples:
        z = ((x - 0x00010001) & ~x) & M32
        if x & M16 == 0:
            assert z & 0x8000
        if x >> 16 == 0:
            assert z & 0x80000000
        # and a word with no zero half is never flagged in its low half
        if x & M16:
            assert not (z & 0x8000) or (x & M16) == 0
