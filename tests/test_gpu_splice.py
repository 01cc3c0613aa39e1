"""GPU parity for the splice-rescue flank DP (split.rs retry_tail_start and
channel A) against the reference's known answers and the oracle."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import oracle as O  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300 import split as S  # noqa: E402
from golden_check import load  # noqa: E402
import workloads as W  # noqa: E402


def _oracle_retry(seq, read, ts, start, end, minus, sig, sup):
    return O.retry_tail_start(O.Contig(seq), read, ts, start, end, minus, sig, sup)


def _same(gpu, orc):
    if orc is None:
        return gpu is None
    if gpu is None:
        return False
    return (gpu.dro, gpu.left_win_lo, gpu.total, gpu.left.key(), gpu.right.key()) == \
        (orc.dro, orc.left_win_lo, orc.total, orc.left.key(), orc.right.key())


@pytest.mark.parametrize("case", load()["retry"], ids=lambda c: c["name"])
def test_retry_known_answers(case):
    g = S.Genome.from_sequences([case["contig"]])
    s, e, minus = case["junction"]
    out = S.retry_tail_start(g, case["read"], case["tail_start"], S.Junction(0, s, e, minus),
                             S.SIG_GTAG, case["support"])
    exp = case["expect"]
    if exp is None:
        assert out is None
    else:
        assert out is not None
        assert out.left.read_end == out.dro
        assert out.right.read_start == exp["right_read_start"]
        assert out.right.ref_start == exp["right_ref_start"]
    orc = _oracle_retry(case["contig"], case["read"], case["tail_start"], s, e, minus,
                        O.SIG_GTAG, case["support"])
    assert _same(out, orc)


def _rand_contig(rng, n, n_runs=0):
    s = bytearray(rng.choice(b"ACGT") for _ in range(n))
    for _ in range(n_runs):
        a = rng.randrange(n)
        for k in range(a, min(n, a + rng.randrange(1, 6))):
            s[k] = ord("N")
    return bytes(s)


def test_retry_random_vs_oracle():
    rng = random.Random(31)
    for rep in range(120):
        exon1, intron, exon2 = rng.randrange(10, 260), rng.randrange(30, 400), rng.randrange(10, 260)
        seq = bytearray(_rand_contig(rng, exon1 + intron + exon2, n_runs=rep % 4))
        d0, a0 = exon1, exon1 + intron
        seq[d0:d0 + 2] = rng.choice([b"GT", b"GC", b"AT", b"CT", b"AA"])
        seq[a0 - 2:a0] = rng.choice([b"AG", b"AC", b"GC", b"AT", b"TT"])
        seq = bytes(seq)
        L = rng.randrange(8, 200)
        b = rng.randrange(1, L)
        src = seq[max(0, d0 - b):d0] + seq[a0:a0 + (L - b)]
        read = bytearray(src + b"A" * (L - len(src)))
        for _ in range(rng.randrange(0, 4)):
            read[rng.randrange(L)] = rng.choice(b"ACGTN")
        read = bytes(read)
        ts = max(0, b + rng.randrange(-4, 5))
        start = d0 + rng.randrange(-3, 4)
        end = a0 + rng.randrange(-3, 4)
        minus = rng.random() < 0.3
        sig, sup = rng.randrange(4), rng.randrange(0, 12)
        g = S.Genome.from_sequences([seq])
        got = S.retry_tail_start(g, read, ts, S.Junction(0, start, end, minus), sig, sup)
        want = _oracle_retry(seq, read, ts, start, end, minus, sig, sup)
        assert _same(got, want), rep


def _oracle_channel_a(garena, contigs, rarena, reads, cands, r):
    R = reads[r]
    C = contigs[R["contig"]]
    seq = B._ASCII[B.unpack_codes(garena, int(C["base"]), int(C["len"]))].tobytes()
    read = B._ASCII[B.unpack_codes(rarena, int(R["read_pos"]), int(R["read_len"]))].tobytes()
    cs = cands[int(R["cand_first"]):int(R["cand_first"]) + int(R["cand_count"])]
    return O.channel_a(O.Contig(seq), read, int(R["tail_start"]), bool(R["minus"]),
                       [(int(c["start"]), int(c["end"]), bool(c["minus_strand"])) for c in cs],
                       [int(c["support"]) for c in cs])


def test_split_read_subset_channel_a():
    garena, contigs, rarena, reads, cands = W.synth_splice(4, 600)
    g = S.Genome(garena, contigs)
    out, cig, cells = S.channel_a_batch(g, reads, rarena, cands)
    assert cells > 0
    assert (out["status"] == 0).all()
    n_found = 0
    for r in range(len(reads)):
        want = _oracle_channel_a(garena, contigs, rarena, reads, cands, r)
        o = out[r]
        if want is None:
            assert not o["found"], r
            continue
        n_found += 1
        got = (int(o["cand"]), int(o["dro"]), int(o["pos"]), int(o["score"]), int(o["signal"]),
               B.cigar_of(cig[r], int(o["n_ops"])))
        assert got == (want.cand, want.dro, want.pos, want.score, want.signal, want.cigar), r
    assert n_found > len(reads) // 2


def test_score_tail_win_vs_oracle():
    """splice.rs:667-684: score_tail_win is extend_hint at offset 0; tail_gate
    (splice.rs:705-708) on its result."""
    rng = random.Random(0x7A11)
    n = 0
    for _ in range(300):
        tl = rng.randint(0, 60)
        tail = "".join(rng.choice("ACGTN" if rng.random() < 0.1 else "ACGT") for _ in range(tl))
        wl = tl + rng.randint(0, 40)
        win = list("".join(rng.choice("ACGT") for _ in range(wl)))
        k = rng.randint(0, max(0, wl - tl))
        for q in range(min(tl, wl - k)):  # plant the tail with a few edits
            if rng.random() > 0.05:
                win[k + q] = tail[q] if tail[q] != "N" else "A"
        win = "".join(win)
        d = rng.choice([0, 1, 2])
        got = S.score_tail_win(tail, win, S.ExtendParams(edit_dir=d))
        want = O.extend_hint(tail, win, O.Params(edit_dir=d), offset=0)
        assert got.key() == want.key(), (tail, win, d)
        gate = want.read_end - want.read_start
        assert S.tail_gate(got, tl) == (gate * 5 >= tl * 4 and want.score > 0)
        n += 1
    assert n == 300


def test_genome_from_paidx_matches_sequences():
    """A genome loaded from a paidx v1 index (contigs byte-aligned in the
    arena) gives the same retries as one built from the sequences."""
    from paidx_writer import encode
    rng = random.Random(0xDA1D)
    contigs = [_rand_contig(rng, n, 3) for n in (1203, 5001, 777)]
    raw = encode([(f"c{k}", s) for k, s in enumerate(contigs)])
    g1 = S.Genome.from_paidx(raw)
    g2 = S.Genome.from_sequences(contigs)
    n = 0
    for _ in range(60):
        c = rng.randrange(len(contigs))
        seq = contigs[c]
        start = rng.randrange(200, len(seq) - 300)
        end = start + rng.randrange(60, 250)
        b = rng.randrange(20, 130)
        read = seq[start - b:start] + seq[end:end + 150 - b]
        j = S.Junction(c, start, end, rng.random() < 0.3)
        a1 = S.retry_tail_start(g1, read, b, j, S.SIG_GTAG, 3)
        a2 = S.retry_tail_start(g2, read, b, j, S.SIG_GTAG, 3)
        assert (a1 is None) == (a2 is None)
        if a1 is not None:
            assert (a1.dro, a1.left_win_lo, a1.total, a1.left.key(), a1.right.key()) == \
                (a2.dro, a2.left_win_lo, a2.total, a2.left.key(), a2.right.key())
            n += 1
    assert n > 10


def test_align_spliced_vs_oracle():
    """align_spliced on given exon slices (pseudo-reference gathered on the
    device, extend_hint, stitch_cigar, genomic_start) against the oracle."""
    rng = random.Random(0x5E11)
    seqs = [_rand_contig(rng, n, 8) for n in (30000, 12000)]
    g = S.Genome.from_sequences(seqs)
    oc = [O.Contig(s) for s in seqs]
    reads, cs, exl = [], [], []
    for _ in range(400):
        c = rng.randrange(2)
        L = len(seqs[c])
        k = rng.randrange(1, 5)
        pos, exons = rng.randrange(100, 2000), []
        for _ in range(k):  # ascending, disjoint slices with introns between
            ln = rng.randrange(15, 90)
            exons.append((pos, pos + ln))
            pos += ln + rng.randrange(1, 3000)
        if exons[-1][1] > L:
            continue
        body = bytearray(b"".join(seqs[c][s:e] for s, e in exons))
        for q in range(len(body)):  # errors and N
            if rng.random() < 0.03:
                body[q] = rng.choice(b"ACGTN")
        lo, hi = rng.randrange(0, 8), rng.randrange(0, 8)
        read = bytes(body[lo:len(body) - hi]) or b"A"
        reads.append(read)
        cs.append(c)
        exl.append(exons)
    out, ecig, scig = S.align_spliced_batch(g, reads, cs, exl, cigar_stride=256)
    assert (out["status"] == 0).all()
    for k in range(len(reads)):
        ext, st, gs = O.align_spliced_exons(oc[cs[k]], reads[k], exl[k])
        o = out[k]
        x = o["ext"]
        got = (int(x["score"]), int(x["read_start"]), int(x["read_end"]), int(x["ref_start"]),
               tuple(B.cigar_of(ecig[k], int(x["n_ops"]))))
        assert got == ext.key(), (k, exl[k])
        assert list(scig[k][:int(o["n_ops"])]) == st, (k, exl[k])
        assert int(o["genomic_start"]) == gs
    assert len(reads) > 300
