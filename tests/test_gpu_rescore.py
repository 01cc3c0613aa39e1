"""GPU parity of the strict rescoring kernel (align.rs:1060-1165
rescore_with) against the oracle, on random placements over a genome with N
runs, planted and known introns, N / lowercase query bases, and placements
running past the contig end."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import oracle as O  # noqa: E402
from esperanto_gb300 import rescore as R  # noqa: E402
from esperanto_gb300 import split as S  # noqa: E402

from test_rescore_oracle import REF  # noqa: E402


def _contig(rng, n):
    s = bytearray(rng.choice(b"ACGT") for _ in range(n))
    for _ in range(n // 500):
        a = rng.randrange(n)
        for k in range(a, min(n, a + rng.randrange(1, 30))):
            s[k] = ord("N")
    for _ in range(n // 400):  # plant GT..AG / CT..AC motifs
        a = rng.randrange(n - 3000)
        L = rng.randrange(30, 2500)
        if rng.random() < 0.5:
            s[a:a + 2], s[a + L - 2:a + L] = b"GT", b"AG"
        else:
            s[a:a + 2], s[a + L - 2:a + L] = b"CT", b"AC"
    return bytes(s)


def _placement(rng, seq):
    pos = rng.randrange(len(seq))
    ops, q, rf = [], bytearray(), pos
    for _ in range(rng.randrange(1, 7)):
        kind = rng.choices("MIDNS", [6, 1, 1, 1.5, 0.7])[0]
        n = rng.randrange(1, 40) if kind != "N" else rng.choice([rng.randrange(1, 80),
                                                                  rng.randrange(80, 3000),
                                                                  1000, 100, 10])
        ops.append((kind, n))
        if kind == "M":
            for k in range(n):
                b = seq[rf + k] if rf + k < len(seq) else ord("A")
                r = rng.random()
                if r < 0.05:
                    b = rng.choice(b"ACGTNacgtn")
                elif b == ord("N"):
                    b = rng.choice(b"ACGT")
                q.append(b)
            rf += n
        elif kind in "IS":
            q.extend(rng.choice(b"ACGT") for _ in range(n))
        else:
            rf += n
    if rng.random() < 0.1:
        q = q[:max(0, len(q) - rng.randrange(1, 10))]  # query shorter than the CIGAR
    return pos, ops, bytes(q)


def test_rescore_batch_vs_oracle():
    rng = random.Random(0x5C0E)
    seqs = [_contig(rng, n) for n in (20000, 7000, 35000)] + [REF.encode()]
    g = S.Genome.from_sequences(seqs)
    contigs = [O.Contig(s) for s in seqs]
    places = []
    for _ in range(3000):
        c = rng.randrange(len(seqs))
        pos, ops, q = _placement(rng, seqs[c])
        places.append((c, pos, ops, q, rng.choice([0, 1, 2])))
    # a library holding some of the placements' introns (sorted, both strands)
    lib = set()
    for c, pos, ops, q, d in places:
        rf = pos
        for kind, n in ops:
            if kind == "N" and rng.random() < 0.3:
                lib.add((c, rf, rf + n))
            if kind in "MDN":
                rf += n
    lib = sorted(lib)
    L = np.zeros(len(lib), R.LIB_DTYPE)
    for k, (c, s, e) in enumerate(lib):
        L[k] = (c, s, e, k & 1)
    items = np.zeros(len(places), R.RESCORE_ITEM_DTYPE)
    qarena, allops = bytearray(), []
    for k, (c, pos, ops, q, d) in enumerate(places):
        items[k] = (len(qarena), len(q), c, pos, len(allops), len(ops), d)
        qarena += q
        allops += R.encode_cigar(ops)
    out = R.rescore_batch(g, items, np.frombuffer(bytes(qarena), np.uint8),
                          np.array(allops, np.uint32), L)
    assert (out["status"] == 0).all()
    fields = ("score", "aligned", "matches", "mm", "ea_ag", "ea_tc", "ins", "del", "clipped",
              "n_splice", "splice_score")
    n_splice = 0
    for k, (c, pos, ops, q, d) in enumerate(places):
        want = O.rescore(contigs[c], c, pos, q, R.encode_cigar(ops), lib, edit_dir=d)
        got = tuple(int(out[k][f]) for f in fields)
        assert got == want, (k, c, pos, ops, q, d)
        n_splice += got[9]
    assert n_splice > 500


def test_rescore_with_single_placement():
    g = S.Genome.from_sequences([REF])
    s = R.rescore_with(g, "ACTTGC", 0, 4, [("M", 2), ("N", 1000), ("M", 4)])
    assert s.key() == (16, 6, 6, 0, 0, 0, 0, 0, 0, 1, 4)
    s = R.rescore_with(g, "ACTTGC", 0, 4, [("M", 2), ("N", 1000), ("M", 4)],
                       junction_lib=[(0, 6, 1006)])
    assert s.score == 18 and s.splice_score == 6
