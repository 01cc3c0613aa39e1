"""The end trim of the device traceback (gotoh.cu, dp_finish) restated in
Python and checked against the reference's rule (extend.rs:930-962, as the
oracle's extend.c restates it) on random step sequences, the degenerate
keep-the-middle case included.

The reference reverses the walk into forward order, takes `lead` = 1 + the
last forward index whose prefix sum is <= 0 and `trail` = the number of
trailing steps whose suffix sum is <= 0 (extending backwards), keeps
[lead, n - trail), and keeps only the middle step n // 2 when lead + trail
>= n.  The device never reverses: over walk-order prefix sums P_t it takes
its `trail` from the last P_t <= 0, finds u, the first walk index in
[-1, n - 2] with P_u >= T (P_-1 = 0, T = P_{n-1}), from each 8-step block's
prefix sum before it and its largest prefix sum, keeps walk indices
[trail, u] (through n - 1 when no u exists), and degenerates exactly when
T <= 0 or u < trail.
"""
import random

DELTAS = (2, -4, 0, -6, -2)  # match, mismatch, tolerated, gap open, gap extend


def reference_kept(fwd):
    """Kept forward indices [a, b) under extend.rs's rule (extend.c)."""
    n = len(fwd)
    lead = trail = 0
    acc = 0
    for k in range(n):
        acc += fwd[k]
        if acc <= 0:
            lead = k + 1
    acc = 0
    for kk in range(n - 1, -1, -1):
        acc += fwd[kk]
        if acc <= 0:
            trail = n - kk
    degenerate = n > 0 and lead + trail >= n
    if degenerate:
        lead = n // 2
        trail = n - lead - 1
    return lead, n - trail, degenerate


def device_kept(walk):
    """Kept walk indices [lo, hi] the way dp_finish finds them."""
    n = len(walk)
    P, trail = 0, 0
    pst, bmx = [], []
    bm, pb = None, 0
    for t, d in enumerate(walk):
        P += d
        bm = P if bm is None else max(bm, P)
        if (t + 1) % 8 == 0:
            pst.append(pb)
            bmx.append(bm)
            bm, pb = None, P
        if P <= 0:
            trail = t + 1
    if n % 8:
        pst.append(pb)
        bmx.append(bm)
    T = P
    ue, degenerate = n - 1, T <= 0
    if not degenerate:
        for b in range(len(bmx)):
            if bmx[b] < T:
                continue
            Pb = pst[b]
            found = None
            for t in range(8 * b, min(8 * b + 7, n - 2) + 1):
                Pb += walk[t]
                if Pb >= T:
                    found = t
                    break
            if found is not None:
                ue = found
                degenerate = found < trail
            break
    if degenerate:
        tstar = n - 1 - n // 2
        return tstar, tstar
    return trail, ue


def test_record_trim_equals_the_reference_rule():
    rng = random.Random(7)
    seen_degenerate = seen_cut = 0
    for case in range(20000):
        n = rng.randrange(1, 70)
        # mostly alignments that climb, some that wander below zero
        w = [rng.choice(DELTAS) if rng.random() < 0.35 else 2 for _ in range(n)]
        if case % 5 == 0:
            w = [rng.choice(DELTAS) for _ in range(n)]
        walk = w  # walk order: from the best cell backwards
        fwd = walk[::-1]
        a, b, degenerate = reference_kept(fwd)
        lo, hi = device_kept(walk)
        # walk index t is forward index n - 1 - t
        assert (n - 1 - hi, n - hi + (hi - lo)) == (a, b), (walk, a, b, lo, hi)
        seen_degenerate += degenerate
        seen_cut += degenerate and sum(walk) > 0  # u < trail, not T <= 0
    # the keep-the-middle case was exercised, both by T <= 0 and by u < trail
    assert seen_degenerate > 100 and seen_cut > 100
