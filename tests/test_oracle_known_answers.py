"""Pin the CPU oracle against the reference's own known answers
(crates/map/src/extend.rs:2033-2571, crates/map/src/split.rs:962-1029)."""
import pytest

import oracle as O
from golden_check import check_extension, load

G = load()


def _params(d):
    return O.Params(**d)


def run_kind(kind, case):
    p = _params(case["params"])
    band = tuple(case["band"]) if case.get("band") is not None else None
    r, w = case["read"], case["window"]
    if kind == "run_band_i16":
        return O.run_band(r, w, p, wide=False, band=band)[0]
    if kind == "run_band_i32":
        return O.run_band(r, w, p, wide=True, band=band)[0]
    if kind == "run_dispatch":
        return O.run_dispatch(r, w, p, band=band)[0]
    if kind == "extend":
        return O.extend(r, w, p)
    if kind == "extend_hint":
        return O.extend_hint(r, w, p, offset=case.get("offset", 0))
    raise AssertionError(kind)


def test_extension_known_answers():
    groups = {}
    for case in G["extension"]:
        for kind in case["kinds"]:
            ext = run_kind(kind, case)
            check_extension(ext, case["expect"], f"{case['name']} [{kind}]")
            g = case["expect"].get("cigar_group")
            if g is not None:
                groups.setdefault(g, []).append(tuple(ext.cigar))
    # every kernel flavour yields the same CIGAR on each input (:2120-2121)
    for g, cigs in groups.items():
        assert len(set(cigs)) == 1, (g, cigs)


@pytest.mark.parametrize("case", G["retry"], ids=lambda c: c["name"])
def test_retry_known_answers(case):
    ctg = O.Contig(case["contig"])
    s, e, minus = case["junction"]
    sig = {"GtAg": O.SIG_GTAG}[case["signal"]]
    out = O.retry_tail_start(ctg, case["read"], case["tail_start"], s, e, minus, sig,
                             case["support"])
    exp = case["expect"]
    if exp is None:
        assert out is None, out
    else:
        assert out is not None
        assert out.left.read_end == out.dro
        assert out.right.read_start == exp["right_read_start"]
        assert out.right.ref_start == exp["right_ref_start"]


def test_i16_sentinel_clamp():
    # extend.rs:2441-2458
    for a, b, want in G["i16_add"]:
        assert O.i16_add(a, b) == want
