"""Write tests/golden/known_answers.json: the literal known answers of the
reference's own unit tests for the hot path, as replayable cases.

Each case restates how one reference test builds its inputs and what it
asserts (file:line in the case's "ref" field).  Expected values are the
reference's literals, never outputs of this repository's code, so the
fixture pins both the oracle and the GPU path.

Run:  python tests/golden/make_known_answers.py
"""
from __future__ import annotations

import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from refgen import body, revcomp  # noqa: E402

OFF, AG, TC = 0, 1, 2
DEFAULT = dict(match_score=2, mismatch=-4, gap_open=4, gap_ext=2, edit_dir=OFF)


def P(**kw):
    d = dict(DEFAULT)
    d.update(kw)
    return d


def s(b: bytes) -> str:
    return b.decode()


cases = []


def add(**kw):
    """One input with the reference kernels it is asserted on ("kinds")."""
    cases.append(kw)


# extend.rs:2033-2128 affine_gap_score_matches_the_common_candidate_domain
reference = body(160)
group = 0
for insertion in (False, True):
    for n in (1, 2, 3, 7):
        query = bytearray(reference)
        if insertion:
            b = next(x for x in b"ACGT" if x != reference[79] and x != reference[80])
            query[80:80] = bytes([b]) * n
        else:
            del query[80:80 + n]
        query = bytes(query)
        for reverse in (False, True):
            q, r = (revcomp(query), revcomp(reference)) if reverse else (query, reference)
            for d in (OFF, AG, TC):
                for offset in (0, 37):
                    window = b"N" * offset + r + b"N" * 11
                    expected_match = len(r) if insertion else len(q)
                    expected = expected_match * 2 - 4 - 2 * n
                    for band in (None, (offset, 30)):
                        group += 1
                        exp = dict(score=expected, read_start=0, read_end=len(q),
                                   ref_start=offset,
                                   cigar_contains=[["I" if insertion else "D", n]],
                                   cigar_group=group)
                        ctx = f"ins={insertion} n={n} rev={reverse} dir={d} off={offset} band={band}"
                        add(name="affine_gap_domain " + ctx,
                            kinds=["run_band_i16", "run_band_i32", "run_dispatch",
                                   "extend_hint"],
                            read=s(q), window=s(window), params=P(edit_dir=d), band=band,
                            offset=offset, expect=exp,
                            ref="crates/map/src/extend.rs:2033-2128")

# extend.rs:2131-2162 affine_gap_terminal_path_cannot_borrow_a_missing_extension_penalty
b120 = body(120)
ref2 = b120 + b"TAGC"
qry2 = b120 + b"AGC" + b"N" * 27
for reverse in (False, True):
    q, r = (revcomp(qry2), revcomp(ref2)) if reverse else (qry2, ref2)
    add(name=f"terminal_path rev={reverse}", kinds=["extend"], read=s(q), window=s(r), params=P(),
        expect=dict(score=240, no_gaps=True), ref="crates/map/src/extend.rs:2131-2162")

# extend.rs:2165-2180 affine_gap_rescue_penalties_keep_an_ungapped_local_body
q3 = bytearray(reference)
del q3[80]
add(name="rescue_penalties_400", kinds=["extend"], read=s(bytes(q3)), window=s(reference),
    params=P(gap_open=400, gap_ext=400), expect=dict(score_positive=True, no_gaps=True),
    ref="crates/map/src/extend.rs:2165-2180")

core = b"GACGATCGGATACGCTAGCA"
# extend.rs:2183-2226 neutral_outer_flanks_keep_edit_evidence_without_score_gain
for rf, qf in ((b"AAT", b"AAC"), (b"CCA", b"CCG")):
    for left in (True, False):
        r, q = bytearray(b"NN"), bytearray()
        if left:
            r += rf
            q += b"NN" + qf
        r += core
        q += core
        if not left:
            r += rf[::-1]
            q += qf[::-1] + b"NN"
        r += b"NN"
        add(name=f"neutral_flanks_edit_evidence {rf} left={left}", kinds=["extend_hint"],
            read=s(bytes(q)), window=s(bytes(r)), params=P(), offset=0 if left else 2,
            expect=dict(score=40, ref_start=2,
                        cigar=[["S", 2], ["M", 23]] if left else [["M", 23], ["S", 2]]),
            ref="crates/map/src/extend.rs:2183-2226")

# extend.rs:2229-2250 neutral_outer_flanks_do_not_absorb_negative_or_ambiguous_clips
r5 = b"AATGACGATCGGATACGCTAGCA"
for prefix in (b"NNN", b"ACC"):
    add(name=f"neutral_no_absorb {prefix}", kinds=["extend_hint"], read=s(prefix + r5[3:]),
        window=s(r5), params=P(), offset=0,
        expect=dict(score=40, read_start=3, ref_start=3, cigar=[["S", 3], ["M", 20]]),
        ref="crates/map/src/extend.rs:2229-2250")


def exempt_dir(ref_b, read_b):
    if (ref_b, read_b) == (ord("A"), ord("G")):
        return True
    if (ref_b, read_b) == (ord("T"), ord("C")):
        return False
    return None


# extend.rs:2253-2319 neutral_non_n_technical_tails_do_not_buy_coverage...
tails = [b"AGATCGGAAGAGCACACGTCTGAACTCCAGTCA", b"AAAAAAAAAAAAAAAAAAAA", b"CAGTCGTACGATCTAG"]
for tail in tails:
    for left in (True, False):
        flank = bytearray(tail[-3:] if left else tail[:3])
        mm = 2 if left else 0
        edge = tail[-1] if left else tail[0]
        flank[mm] = next(x for x in b"ACGT" if x != flank[mm] and exempt_dir(x, edge) is None)
        pad = len(tail) + 2
        r, q = bytearray(b"N" * pad), bytearray()
        if left:
            r += flank
            q += tail
        r += core
        q += core
        if not left:
            r += flank
            q += tail
        r += b"N" * pad
        for d in (OFF, AG, TC):
            for lower in (False, True):
                rr, qq = bytes(r), bytes(q)
                if lower:
                    rr, qq = rr.lower(), qq.lower()
                add(name=f"technical_tail {tail[:6]} left={left} dir={d} lower={lower}",
                    kinds=["extend"], read=s(qq), window=s(rr), params=P(edit_dir=d),
                    expect=dict(score=40, ref_start=pad + (3 if left else 0),
                                cigar=[["S", len(tail)], ["M", 20]] if left
                                else [["M", 20], ["S", len(tail)]]),
                    ref="crates/map/src/extend.rs:2253-2319")

# extend.rs:2322-2341 neutral_flank_scan_does_not_cross_an_ordinary_mismatch...
add(name="neutral_scan_no_cross", kinds=["extend"], read=s(b"NNAAGAAC" + core),
    window=s(b"NNAATAAT" + core), params=P(),
    expect=dict(score=40, read_start=5, ref_start=5, cigar=[["S", 5], ["M", 23]]),
    ref="crates/map/src/extend.rs:2322-2341")

# extend.rs:2344-2390 terminal_edit_ties_survive_all_edit_modes_and_scalar_dispatch
for rf, qf, direction in ((b"AAT", b"AAC", TC), (b"CCA", b"CCG", AG)):
    for left in (True, False):
        for d in (OFF, AG, TC):
            for lower in (False, True):
                r, q = bytearray(b"NN"), bytearray(b"NN")
                if left:
                    r += rf
                    q += qf
                r += core
                q += core
                if not left:
                    r += rf[::-1]
                    q += qf[::-1]
                r += b"NN"
                q += b"NN"
                rr, qq = bytes(r), bytes(q)
                if lower:
                    rr, qq = rr.lower(), qq.lower()
                add(name=f"terminal_edit_ties {rf} left={left} dir={d} lower={lower}",
                    kinds=["extend"], read=s(qq), window=s(rr), params=P(edit_dir=d),
                    expect=dict(score=40 + (4 if d == direction else 0), ref_start=2,
                                cigar=[["S", 2], ["M", 23], ["S", 2]]),
                    ref="crates/map/src/extend.rs:2344-2390")

# extend.rs:2393-2414 identical_edit_and_technical_origin_sequences_remain_indistinguishable
add(name="identical_edit_technical", kinds=["extend"], read="NNAACGACGATCGGATACGCTAGCA",
    window="NNAATGACGATCGGATACGCTAGCA", params=P(),
    expect=dict(cigar=[["S", 2], ["M", 23]]), ref="crates/map/src/extend.rs:2393-2414")

# extend.rs:2417-2435 positive_score_ordinary_terminal_alignment_is_not_a_neutral_tie
add(name="positive_ordinary_terminal", kinds=["extend"], read=s(b"NNAAAA" + core),
    window=s(b"NNAAAC" + core), params=P(),
    expect=dict(score=42, cigar=[["S", 2], ["M", 24]]), ref="crates/map/src/extend.rs:2417-2435")

# extend.rs:2542-2571 full_matrix_short_reference_covers_late_query_matches
for m, n in ((4, 1), (33, 7), (80, 15), (150, 55), (301, 31)):
    rf = bytes(b"ACGT"[i % 4] for i in range(n))
    read = b"N" * (m - n) + rf
    exp = dict(read_start=m - n, read_end=m, ref_start=0, score=2 * n,
               cigar=[["S", m - n], ["M", n]])
    add(name=f"short_reference m={m} n={n}", kinds=["run_band_i16", "run_band_i32", "extend"],
        read=s(read), window=s(rf), params=P(), band=None, expect=exp,
        ref="crates/map/src/extend.rs:2542-2571")

# crates/map/src/split.rs:962-1029 retry_tail_start (junction 60 -> 160, GT-AG,
# support 2, default parameters)
seq_ok = "A" * 20 + "C" * 40 + "GT" + "T" * 96 + "AG" + "G" * 60
retry = []
retry.append(dict(name="retry_rejects_internal_seam_clip", contig=seq_ok,
                  read="C" * 40 + "AAAA" + "G" * 40, tail_start=44, expect=None,
                  ref="crates/map/src/split.rs:962-979"))
retry.append(dict(name="retry_rejects_gap_before_donor",
                  contig="A" * 20 + "C" * 36 + "AAAAGT" + "T" * 96 + "AG" + "G" * 60,
                  read="C" * 40 + "G" * 40, tail_start=40, expect=None,
                  ref="crates/map/src/split.rs:982-997"))
retry.append(dict(name="retry_rejects_gap_after_acceptor",
                  contig="A" * 20 + "C" * 40 + "GT" + "T" * 96 + "AGAAAA" + "G" * 60,
                  read="C" * 40 + "G" * 40, tail_start=40, expect=None,
                  ref="crates/map/src/split.rs:1000-1015"))
for prefix, suffix in (("", ""), ("TTTT", "AAAA")):
    retry.append(dict(name=f"retry_keeps_exact_splice prefix={prefix!r}", contig=seq_ok,
                      read=prefix + "C" * 40 + "G" * 40 + suffix,
                      tail_start=len(prefix) + 40,
                      expect=dict(left_read_end_is_dro=True, right_read_start=0,
                                  right_ref_start=0),
                      ref="crates/map/src/split.rs:1018-1029"))
for r in retry:
    r.update(junction=[60, 160, False], signal="GtAg", support=2)

out = dict(
    about="Literal known answers of the reference's unit tests for the hot path "
          "(generated by make_known_answers.py; expected values are the reference's).",
    extension=cases,
    retry=retry,
    i16_add=[[-30000, 6, -30000], [-30000, -30000, -30000], [0, -30000, -30000],
             [300, 2, 302], [-31000, -6, -30000]],
)
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
with open(path, "w") as f:
    json.dump(out, f, separators=(",", ":"))
print(f"wrote {len(cases)} extension cases, {len(retry)} retry cases -> {path}")
