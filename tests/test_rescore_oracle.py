"""Oracle of the strict rescoring walk (align.rs:1060-1165 rescore_with):
pinned to the reference's own rescore_strict tests (align.rs:4215-4303),
plus hand-worked known answers of its rules (editing directions, N, clips,
deletions, known and novel introns), and the kernel's intron-length-penalty
table against the host's f64 formula (splice.rs:119-121)."""
import pytest

import oracle as O
from esperanto_gb300 import rescore as R

M = lambda n: (n << 4) | 0  # noqa: E731
I = lambda n: (n << 4) | 1  # noqa: E731,E741
D = lambda n: (n << 4) | 2  # noqa: E731
N = lambda n: (n << 4) | 3  # noqa: E731
S = lambda n: (n << 4) | 4  # noqa: E731

# fields: score aligned matches mm ea_ag ea_tc ins del clipped n_splice splice_score
INTRON = "GT" + "C" * 996 + "AG"  # 1,000-bp intron, GT..AG on the plus strand
REF = "ACGTAC" + INTRON + "TTGCA" + "NNNN" + "ACGT"


@pytest.mark.parametrize("query,pos,ops,edit,lib,want", [
    ("ACGT", 0, [M(4)], 0, (), (8, 4, 4, 0, 0, 0, 0, 0, 0, 0, 0)),
    # ref T / read G: an ordinary mismatch
    ("ACGG", 0, [M(4)], 0, (), (2, 4, 3, 1, 0, 0, 0, 0, 0, 0, 0)),
    # ref A / read G: A-to-G direction; charged unless Ag is exempt
    ("GCGT", 0, [M(4)], 0, (), (2, 4, 3, 0, 1, 0, 0, 0, 0, 0, 0)),
    ("GCGT", 0, [M(4)], 1, (), (6, 4, 3, 0, 1, 0, 0, 0, 0, 0, 0)),
    # ref T / read C under Tc
    ("ACGC", 0, [M(4)], 2, (), (6, 4, 3, 0, 0, 1, 0, 0, 0, 0, 0)),
    # read N and lowercase: N is skipped, lowercase is a plain mismatch
    ("ANGt", 0, [M(4)], 0, (), (0, 3, 2, 1, 0, 0, 0, 0, 0, 0, 0)),
    # 2M 2I 2M: 4 matches, one insertion of 2 (open 4 + 2*2)
    ("ACGGGT", 0, [M(2), I(2), M(2)], 0, (), (0, 6, 4, 0, 0, 0, 1, 0, 0, 0, 0)),
    # 2M 1D 2M over ACGTA: AC, skip G, TA
    ("ACTA", 0, [M(2), D(1), M(2)], 0, (), (2, 5, 4, 0, 0, 0, 0, 1, 0, 0, 0)),
    # 2S 2M: clipped bases advance the read only
    ("TTGT", 2, [S(2), M(2)], 0, (), (4, 2, 2, 0, 0, 0, 0, 0, 2, 0, 0)),
    # novel GT..AG intron of 1,000 bp: +4 motif, penalty 0
    ("ACTTGC", 4, [M(2), N(1000), M(4)], 0, (),
     (16, 6, 6, 0, 0, 0, 0, 0, 0, 1, 4)),
    # the same intron in the library (either strand): +6 known bonus
    ("ACTTGC", 4, [M(2), N(1000), M(4)], 0, ((0, 6, 1006),),
     (18, 6, 6, 0, 0, 0, 0, 0, 0, 1, 6)),
    # reference N run and past the contig end: uncounted
    ("ACGTACGTAA", len(REF) - 8, [M(10)], 0, (), (8, 4, 4, 0, 0, 0, 0, 0, 0, 0, 0)),
])
def test_known_answers(query, pos, ops, edit, lib, want):
    c = O.Contig(REF)
    assert O.rescore(c, 0, pos, query, ops, lib, edit_dir=edit) == want


def test_intron_penalty_table_matches_f64_formula():
    lens = list(range(1, 20001)) + [10 ** k + d for k in range(4, 10) for d in (-1, 0, 1)]
    lens += [int(1.37 ** k) for k in range(20, 71)] + [2 ** 32 - 1]
    for n in lens:
        assert R.intron_length_penalty(n) == O.intron_length_penalty(n), n


def test_pinned_to_the_reference_rescore_strict_tests():
    """align.rs:4215-4303 (rescore_strict_manual_cigars,
    rescore_strict_splice_signal): rescore_strict is rescore_with with no
    exempt direction."""
    f = {k: i for i, k in enumerate(O.STRICT_FIELDS)}
    ref = O.Contig(b"ACGT" * 50)
    read = (b"ACGT" * 13)[:50]
    s = O.rescore(ref, 0, 0, read, [M(50)])
    assert (s[f["score"]], s[f["matches"]], s[f["mm"]], s[f["aligned"]]) == (100, 50, 0, 50)
    r2 = bytearray(read)
    r2[25] = ord("C") if r2[25] == ord("A") else ord("A")
    s = O.rescore(ref, 0, 0, bytes(r2), [M(50)])
    assert (s[f["score"]], s[f["mm"]]) == (49 * 2 - 4, 1)
    r3 = bytearray(read)
    r3[24] = ord("G")  # ref A at 24 ("ACGT" repeats): an A>G editing-type substitution
    s = O.rescore(ref, 0, 0, bytes(r3), [M(50)])
    assert (s[f["score"]], s[f["mm"]]) == (49 * 2 - 4, 0)
    assert s[f["ea_ag"]] + s[f["ea_tc"]] == 1
    ins_read = read[:24] + b"TT" + read[24:48]
    s = O.rescore(ref, 0, 0, ins_read, [M(24), I(2), M(24)])
    assert (s[f["score"]], s[f["ins"]]) == (48 * 2 - (4 + 2 * 2), 1)
    # exon1 | GT + 56 N + AG | exon2; the read spans 20 + 20 exon bases
    exon1 = b"ACGTTGCAAGGCATTACGACCAAGTTACAGGATCCAAGTTGACGTTACAGGCATTAC"
    intron = b"GT" + b"N" * 56 + b"AG"
    exon2 = b"CATGGACTTGAACCTTGACGTACATGGACTTGAACCTTGACGTA"
    seq = exon1 + intron + exon2
    start, e2 = len(exon1) - 20, len(exon1) + len(intron)
    sread = seq[start:len(exon1)] + seq[e2:e2 + 20]
    sc = O.Contig(seq)
    s = O.rescore(sc, 0, start, sread, [M(20), N(len(intron)), M(20)])
    expected = (40 * 2 + O.splice_params_default().gt_ag_bonus
                - O.intron_length_penalty(len(intron)))
    assert (s[f["score"]], s[f["n_splice"]], s[f["aligned"]]) == (expected, 1, 40)


def test_extension_and_rescore_agree_like_the_reference_test():
    """align.rs:2788-2830 (affine_gap_extension_and_common_rescore_agree):
    over a 160-base xorshift reference with an internal insertion or
    deletion of 1, 2, 3 or 7 bases at 80 and, for the editing directions, one
    edit in [15, 40), the full-matrix extension's score equals the strict
    rescore of its own placement under the same direction."""
    state, ref = 0x75BCD15, bytearray()
    for _ in range(160):  # the reference test's generator
        state ^= (state << 13) & ((1 << 64) - 1)
        state ^= state >> 7
        state ^= (state << 17) & ((1 << 64) - 1)
        ref.append(b"ACGT"[state & 3])
    ref = bytes(ref)
    contig = O.Contig(ref)
    checked = 0
    for insertion in (False, True):
        for n in (1, 2, 3, 7):
            q = bytearray(ref)
            if insertion:
                b = next(c for c in b"ACGT" if c != ref[79] and c != ref[80])
                q[80:80] = bytes([b]) * n
            else:
                del q[80:80 + n]
            for edit in (O.EDIT_OFF, O.EDIT_AG, O.EDIT_TC):
                e = bytearray(q)
                if edit != O.EDIT_OFF:
                    frm, to = (b"A", b"G") if edit == O.EDIT_AG else (b"T", b"C")
                    k = next(i for i in range(15, 40) if e[i] == frm[0])
                    e[k] = to[0]
                ext = O.extend(bytes(e), ref, O.Params(edit_dir=edit))
                if edit == O.EDIT_OFF:
                    # the score and gap the reference asserts for this read
                    # mapped (align.rs:2838-2848)
                    assert ext.score == (160 - (0 if insertion else n)) * 2 - 4 - 2 * n
                    assert ("I" if insertion else "D", n) in ext.cigar
                ops = [(ln << 4) | O.OP_CHARS.index(c) for c, ln in ext.cigar]
                s = O.rescore(contig, 0, ext.ref_start, bytes(e), ops, edit_dir=edit)
                assert ext.score == s[0], (insertion, n, edit, ext.cigar)
                checked += 1
    assert checked == 24
