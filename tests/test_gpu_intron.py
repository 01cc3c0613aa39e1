"""GPU parity of the intron-chain fast path (crates/map/src/intron_chain.rs
:392-538 from the best fragment pair on): the EA-Myers breakpoint
refinement, split-read verification, gates, read-aware junction refinement
against the library, pseudo-reference extend_hint and stitched CIGAR of
every read equal the oracle's, field by field, over synthetic two-exon reads
(canonical and non-canonical motifs, both strands, N runs in the genome and
the reads, fragment pairs that fail each gate)."""
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

STRIDE = 64


def _genome(rng, n_contigs=3, length=120_000):
    seqs = []
    for c in range(n_contigs):
        s = bytearray(rng.choice(b"ACGT") for _ in range(length))
        for _ in range(6):  # N runs
            a, w = rng.randrange(1000, length - 1000), rng.randrange(1, 40)
            s[a:a + w] = b"N" * w
        seqs.append(s)
    return seqs


def _mutate(rng, read):
    r = bytearray(read)
    for _ in range(rng.randrange(0, 4)):
        q = rng.randrange(len(r))
        r[q] = rng.choice(b"ACGT")
    if rng.random() < 0.1:
        q = rng.randrange(len(r))
        r[q] = ord("N")
    return bytes(r)


def _cases(seed, n):
    rng = random.Random(seed)
    seqs = _genome(rng)
    reads, items, lib = [], [], {}
    for k in range(n):
        c = rng.randrange(len(seqs))
        s = seqs[c]
        a = rng.randrange(20, 131)          # exon-1 part of the read
        L = 150
        il = int(np.exp(rng.uniform(np.log(60), np.log(50_000))))
        if k % 23 == 0:
            il = rng.choice([10, 108_000])  # outside [20, intron_max]
        e1 = rng.randrange(500, len(s) - il - 1000)
        j0, j1 = e1 + a, e1 + a + il       # intron [j0, j1)
        minus = rng.random() < 0.5
        don, acc = (b"CT", b"AC") if minus else (b"GT", b"AG")
        if k % 7 == 3:
            don = b"GC" if not minus else b"CT"
        if k % 11 != 5:                      # some non-canonical
            s[j0:j0 + 2] = don
            s[j1 - 2:j1] = acc
        read = bytes(s[e1:j0] + s[j1:j1 + (L - a)])
        if k % 19 == 7:  # an unrelated read: verification rejects it
            read = bytes(rng.choice(b"ACGT") for _ in range(L))
        read = _mutate(rng, read)
        jl = rng.randrange(0, 4)
        jr = rng.randrange(0, 4)
        left = (rng.randrange(0, 4), a - jl, 0, 0, rng.randrange(1, 5))
        left = (left[0], left[1], e1 + left[0], e1 + left[1], left[4])
        rq = a + jr
        right = (rq, L - rng.randrange(0, 4), j1 + (rq - a), 0, rng.randrange(0 if k % 13 else 1, 4))
        right = (right[0], right[1], right[2], j1 + (right[1] - a), right[4])
        if k % 17 == 2:  # a gap in the read between the fragments
            left = (left[0], left[1] - 12, left[2], left[3] - 12, left[4])
        ps, pe = j0 + rng.randrange(-2, 3), j1 + rng.randrange(-2, 3)
        reads.append(read)
        items.append((c, left, right, ps, pe, minus))
        if k % 3 == 0:
            lib[(c, j0, j1, int(minus))] = rng.randrange(1, 9)
        if k % 5 == 0:
            lib[(c, j0 + 1, j1 + 1, int(not minus))] = 2
    return seqs, reads, items, sorted(key + (cnt,) for key, cnt in lib.items())


def test_intron_chain_batch_matches_oracle():
    seqs, reads, items, lib = _cases(77, 3000)
    g = S.Genome.from_sequences([bytes(s) for s in seqs])
    arena, pp, n_iv = B.pack_ascii_pairs(reads, [b""] * len(reads), [0] * len(reads),
                                         [0] * len(reads))
    recs = np.zeros(len(reads), S.INTRON_READ_DTYPE)
    for k, (c, left, right, ps, pe, minus) in enumerate(items):
        recs[k]["read_pos"] = pp[k]["read_pos"]
        recs[k]["read_len"] = pp[k]["read_len"]
        recs[k]["contig"] = c
        recs[k]["n_first"] = pp[k]["n_first"]
        recs[k]["n_read"] = pp[k]["n_read"]
        recs[k]["minus"] = int(minus)
        recs[k]["intron_start"], recs[k]["intron_end"] = ps, pe
        recs[k]["left"] = left
        recs[k]["right"] = right
    libarr = np.array(lib, dtype=S.LIB_JUNCTION_DTYPE)
    out, ec, sc = S.intron_chain_batch(g, recs, arena, libarr, n_iv, cigar_stride=STRIDE)
    contigs = [O.Contig(bytes(s)) for s in seqs]
    stages = {}
    for k, (c, left, right, ps, pe, minus) in enumerate(items):
        want = O.intron_chain(contigs[c], c, reads[k], left, right, ps, pe, minus, lib)
        o = out[k]
        ctx = (k, want.stage)
        assert S.IC_STAGES[int(o["stage"])] == want.stage, (ctx, S.IC_STAGES[int(o["stage"])])
        assert bool(o["found"]) == want.found, ctx
        stages[want.stage] = stages.get(want.stage, 0) + 1
        if want.stage == "empty":
            continue
        assert (int(o["donor_end"]), int(o["acceptor_start"])) == (want.donor_end,
                                                                   want.acceptor_start), ctx
        assert (int(o["verify_donor"]), int(o["verify_acceptor"])) == (want.vd, want.va), ctx
        if want.stage in ("anchors", "intron", "verify"):
            continue
        assert (int(o["j_start"]), int(o["j_end"]), bool(o["j_minus"])) == want.junction, ctx
        assert (int(o["signal"]), int(o["support"])) == (want.signal, want.support), ctx
        if want.stage == "junction":
            continue
        assert (int(o["left_start"]), int(o["right_end"])) == (want.left_start,
                                                               want.right_end), ctx
        if want.stage == "bounds":
            continue
        x = o["ext"]
        got = (int(x["score"]), int(x["read_start"]), int(x["read_end"]), int(x["ref_start"]),
               tuple(B.cigar_of(ec[k], int(x["n_ops"]))))
        assert got == want.ext.key(), ctx
        assert B.cigar_of(sc[k], int(o["n_ops"])) == want.cigar, ctx
    # every gate is exercised, and most reads are placed
    for st in ("found", "anchors", "intron", "verify"):
        assert stages.get(st, 0) > 0, stages
    assert stages["found"] > len(items) // 2, stages
