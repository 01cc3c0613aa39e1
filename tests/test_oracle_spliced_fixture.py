"""The oracle's spliced pseudo-reference path (splice.rs:617-664
align_spliced with stitch_cigar; oracle/spliced.c) on the reference's own
try_spliced fixture (align.rs:5588-5640, try_spliced_stitches_two_segment_chain):
57 exon bases, a 60-base GT..AG intron, 44 exon bases, and a 40-base read
spanning the last 20 bases of exon 1 and the first 20 of exon 2.  The
reference expects position 37, CIGAR M20 N60 M20 and a GT-AG junction at
[57, 117).  The chain-to-exon step (prepare_spliced) stays with the caller,
so the exon slices are given: exactly the read's two segments, and padded
ones (the DP then soft-clips nothing and still lands at 37)."""
import oracle as O

EXON1 = "ACGTTGCAAGGCATTACGACCAAGTTACAGGATCCAAGTTGACGTTACAGGCATTAC"
INTRON = "GT" + "N" * 56 + "AG"
EXON2 = "CATGGACTTGAACCTTGACGTACATGGACTTGAACCTTGACGTA"

M = lambda n: (n << 4) | 0  # noqa: E731
N = lambda n: (n << 4) | 3  # noqa: E731


def test_try_spliced_fixture():
    assert len(EXON1) == 57 and len(INTRON) == 60 and len(EXON2) == 44
    seq = (EXON1 + INTRON + EXON2).encode()
    start = len(EXON1) - 20
    e2 = len(EXON1) + len(INTRON)
    read = seq[start:len(EXON1)] + seq[e2:e2 + 20]
    contig = O.Contig(seq)
    for exons in ([(37, 57), (117, 137)], [(27, 57), (117, 147)], [(0, 57), (117, 161)]):
        ext, stitched, gstart = O.align_spliced_exons(contig, read, exons)
        assert gstart == 37, (exons, gstart)
        assert stitched == [M(20), N(60), M(20)], (exons, stitched)
        assert ext.score == 40 * 2
    assert O.junction_signal(contig, 57, 117, False) == O.SIG_GTAG
