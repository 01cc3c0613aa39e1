"""Shared checks of an extension result against the reference's literal
known answers (tests/golden/known_answers.json)."""
import json
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers.json")


def load():
    with open(GOLDEN) as f:
        return json.load(f)


def check_extension(ext, expect, ctx=""):
    """`ext` has score/read_start/read_end/ref_start and cigar [(op, len)]."""
    cig = [(op, n) for op, n in ext.cigar]
    for key in ("score", "read_start", "read_end", "ref_start"):
        if key in expect:
            assert getattr(ext, key) == expect[key], f"{key} {ctx}: {ext}"
    if "cigar" in expect:
        assert cig == [(op, n) for op, n in expect["cigar"]], f"cigar {ctx}: {cig}"
    for op, n in expect.get("cigar_contains", []):
        assert (op, n) in cig, f"cigar lacks {op}{n} {ctx}: {cig}"
    if expect.get("no_gaps"):
        assert not any(op in "ID" for op, _ in cig), f"gapped {ctx}: {cig}"
    if expect.get("score_positive"):
        assert ext.score > 0, ctx
