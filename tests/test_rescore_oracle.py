"""Oracle of the strict rescoring walk (align.rs:1060-1165 rescore_with):
hand-worked known answers from the reference's rules (the reference has no
direct test of rescore_with), and the kernel's intron-length-penalty table
against the host's f64 formula (splice.rs:119-121)."""
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
