"""stitch_cigar (splice.rs:435-493) in the oracle against the reference's own
expectations (crates/map/tests/splice_stitch.rs:41-141)."""
import pytest

import oracle as O

M = lambda n: (n << 4) | 0  # noqa: E731
I = lambda n: (n << 4) | 1  # noqa: E731,E741
D = lambda n: (n << 4) | 2  # noqa: E731
N = lambda n: (n << 4) | 3  # noqa: E731
S = lambda n: (n << 4) | 4  # noqa: E731

TWO = [(0, 100, 110), (10, 210, 230)]
THREE = [(0, 100, 110), (10, 210, 220), (20, 420, 440)]


def spans(ops):
    q = r = 0
    for o in ops:
        n, c = o >> 4, o & 15
        assert n > 0  # never a zero-length op
        if c == 0:
            q += n
            r += n
        elif c in (1, 4):
            q += n
        else:
            r += n
    return q, r


@pytest.mark.parametrize("inp,want", [  # splice_stitch.rs:41-83 (both strands alike)
    ([M(10), I(1), M(10)], [M(10), I(1), N(100), M(10)]),
    ([M(10), D(2), M(8)], [M(10), N(100), D(2), M(8)]),
    ([M(8), D(2), M(10)], [M(8), D(2), N(100), M(10)]),
    ([M(8), D(2), I(1), M(10)], [M(8), D(2), I(1), N(100), M(10)]),
    ([S(3), M(10), I(1), M(10), S(2)], [S(3), M(10), I(1), N(100), M(10), S(2)]),
])
def test_exon_boundary_resumption(inp, want):
    got = O.stitch_cigar(inp, 0, TWO, [100])
    assert got == want
    q, r = spans(inp)
    assert spans(got) == (q, r + 100)


def test_multiple_boundaries():  # splice_stitch.rs:85-116
    inp = [S(3), M(10), I(1), M(10), D(2), M(8), S(2)]
    got = O.stitch_cigar(inp, 0, THREE, [100, 200])
    assert got == [S(3), M(10), I(1), N(100), M(10), N(200), D(2), M(8), S(2)]
    q, r = spans(inp)
    assert spans(got) == (q, r + 300)


@pytest.mark.parametrize("start,inp,want", [  # splice_stitch.rs:118-141
    (0, [M(20)], [M(10), N(100), M(10)]),
    (8, [D(4), M(6)], [D(2), N(100), D(2), M(6)]),
    (0, [M(10), I(1)], [M(10), I(1)]),
    (10, [I(1), M(10)], [I(1), M(10)]),
    (11, [M(5)], [M(5)]),
    (0, [M(8)], [M(8)]),
])
def test_offsets_and_non_crossing(start, inp, want):
    got = O.stitch_cigar(inp, start, TWO, [100])
    assert got == want
    spans(got)


def test_no_bounds_is_identity():
    inp = [M(5), I(1), M(5)]
    assert O.stitch_cigar(inp, 0, [], []) == inp


def test_align_spliced_exons_round_trip():
    """A read spanning three exons aligns end to end on the pseudo-reference
    and stitches back to M/N runs of the exon lengths."""
    import random
    rng = random.Random(7)
    g = "".join(rng.choice("ACGT") for _ in range(3000))
    exons = [(100, 160), (700, 750), (1900, 1990)]
    read = "".join(g[s:e] for s, e in exons)[10:-15]
    ext, st, gs = O.align_spliced_exons(O.Contig(g), read, exons)
    assert ext.score == 2 * len(read)
    assert st == [M(50), N(540), M(50), N(1150), M(75)]
    assert gs == 110
