"""Oracle self-consistency on the reference's seeded sweeps.

The reference's sweeps (crates/map/src/extend.rs:2578-2913) pin its AVX2
kernels to the i16 scalar kernel.  Here the same inputs pin the i16 and i32
flavours of the restated scalar kernel to each other (the reference's
run_dispatch routes pure input to i16 and anything else to i32 and promises
identical Extensions), and the Myers restatements to a brute-force DP.
"""
import random

import pytest

import oracle as O
import refgen as R


def test_full_matrix_sweep_i16_equals_i32():
    n_cases = 0
    for read, win, d, ctx in R.sweep_full_matrix():
        p = O.Params(edit_dir=d)
        a, ta = O.run_band(read, win, p, wide=False)
        b, tb = O.run_band(read, win, p, wide=True)
        assert a.key() == b.key(), ctx
        assert ta == tb, ctx
        n_cases += 1
    assert n_cases > 300


def test_full_block_boundaries_i16_equals_i32():
    for read, win, d, ctx in R.sweep_full_block_boundaries():
        p = O.Params(edit_dir=d)
        assert O.run_band(read, win, p)[0].key() == O.run_band(read, win, p, wide=True)[0].key(), ctx


def test_band_sweep_i16_equals_i32():
    n_cases = 0
    for read, win, d, off, half, ctx in R.sweep_band():
        p = O.Params(edit_dir=d)
        a, ta = O.run_band(read, win, p, wide=False, band=(off, half))
        b, tb = O.run_band(read, win, p, wide=True, band=(off, half))
        assert a.key() == b.key(), ctx
        assert ta == tb, ctx
        n_cases += 1
    assert n_cases > 500


def test_band_block_boundaries_i16_equals_i32():
    for read, win, d, off, half, ctx in R.sweep_band_block_boundaries():
        p = O.Params(edit_dir=d)
        a = O.run_band(read, win, p, band=(off, half))
        b = O.run_band(read, win, p, wide=True, band=(off, half))
        assert a[0].key() == b[0].key() and a[1] == b[1], ctx


def test_empty_inputs():
    # extend.rs:2624-2625 degenerate shapes; :430-442 empty_extension
    assert O.run_band(b"", b"ACGT")[0].key() == (0, 0, 0, 0, ())
    assert O.run_band(b"ACGT", b"")[0].key() == (0, 0, 0, 0, (("S", 4),))
    assert O.extend_hint(b"ACGT", b"").key() == (0, 0, 0, 0, (("S", 4),))


def test_cigar_conserves_read_length():
    rng = R.Rng(7)
    for m, n in [(20, 60), (150, 214), (5, 3), (100, 40)]:
        for _ in range(20):
            read = R.rand_seq(rng, m)
            win = R.rand_window(rng, read, n)
            e = O.extend_hint(read, win, O.Params(), offset=(n - m) // 2)
            assert sum(k for op, k in e.cigar if op in "MIS") == m


def _rand_dna(rng, n, alphabet="ACGT"):
    return bytes(rng.choice(alphabet.encode()) for _ in range(n))


@pytest.mark.parametrize("m", [1, 2, 63, 64, 65, 127, 128, 129, 150, 255, 256])
def test_myers_matches_bruteforce(m):
    rng = random.Random(1000 + m)
    for rep in range(12):
        n = rng.choice([0, 1, m // 2 + 1, m, m + 40, 2 * m + 7])
        text = _rand_dna(rng, n, "ACGTacgtN" if rep % 3 == 0 else "ACGT")
        if n >= m and rep % 2 == 0:
            start = rng.randrange(0, n - m + 1)
            read = bytearray(text[start:start + m].upper().replace(b"N", b"A"))
            for _ in range(rng.randrange(0, 6)):
                read[rng.randrange(m)] = rng.choice(b"ACGTN")
            read = bytes(read)
        else:
            read = _rand_dna(rng, m, "ACGTN" if rep % 4 == 1 else "ACGT")
        want = O.ea_edit_dp(read, text)
        got = O.myers_long_infix_best_end(read, text)
        assert got == want, (m, n, rep)
        if m <= 128:
            assert O.myers_infix_best_end(read, text) == want
            assert O.myers_infix(read, text) == want[0]
        assert O.myers_long_infix(read, text) == want[0]
        # crates/engine/src/myers.rs formulation agrees on the distance
        assert O.engine_infix(read, text) == want[0]
        # best_start = best_end on the reversed pair (myers_ea.rs:158-185)
        rd, rend = O.ea_edit_dp(read[::-1], text[::-1])
        assert O.myers_long_infix_best_start(read, text) == (rd, n - rend)


def test_myers_guards():
    # m = 0 -> (0, 0); m > 256 -> (m, 0) (myers_ea.rs:118-156)
    assert O.myers_infix_best_end(b"", b"ACGT") == (0, 0)
    assert O.myers_long_infix_best_end(b"A" * 300, b"ACGT") == (300, 0)
    with pytest.raises(O.OracleError):
        O.myers_infix_best_end(b"A" * 150, b"ACGT")  # single-block entry, 128 < m
    with pytest.raises(O.OracleError):
        O.engine_infix(b"", b"ACGT")  # MyersEa::new asserts 1 <= m


def test_engine_global_matches_dp():
    rng = random.Random(5)
    for _ in range(200):
        m = rng.randrange(1, 257)
        n = rng.randrange(0, 300)
        read = _rand_dna(rng, m)
        text = _rand_dna(rng, n)
        # global EA distance: D[0][j] = j, D[i][0] = i
        prev = list(range(n + 1))
        for i in range(1, m + 1):
            cur = [i] + [0] * n
            for j in range(1, n + 1):
                free = O.ea_edit_dp(read[i - 1:i], text[j - 1:j])[0] == 0
                cur[j] = min(prev[j - 1] + (0 if free else 1), prev[j] + 1, cur[j - 1] + 1)
            prev = cur
        assert O.engine_global(read, text) == prev[n]
        if _ > 20:
            break
