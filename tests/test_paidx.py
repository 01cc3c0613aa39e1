"""paidx v1 contig reader (index_io.rs decode_parts): layout, strict
validation with the reference's messages, and the genome layout it yields.
Host-only (no device calls)."""
import struct

import numpy as np
import pytest

from esperanto_gb300 import batch as B
from esperanto_gb300 import split as S
from paidx_writer import encode, pack_contig

SEQS = [("chr1", "ACGTACGTTGCAAGCTNNNNACGTAC"), ("chrM", "GATTACA"),
        ("chrUn", "nnACGTRYacgt"), ("empty", "")]
TABLES = dict(kmers=[3, 9, 40], offsets=[0, 2, 3], counts=[2, 1, 1], positions=[5, 7, 1, 0])


def test_contigs_roundtrip_and_layout():
    raw = encode(SEQS, **TABLES)
    info = S.paidx_scan(raw)
    assert (info.k, info.w, info.contig_count, info.kmer_count, info.positions_count) == \
        (5, 2, 4, 3, 4)
    arena, contigs, iv, names, _ = S.paidx_contigs(raw)
    assert names == [n for n, _ in SEQS]
    codes = B.unpack_codes(arena, 0, len(arena) * 4)
    for c, (name, seq) in enumerate(SEQS):
        rec = contigs[c]
        assert rec["base"] % 4 == 0 and rec["len"] == len(seq)
        packed, runs = pack_contig(seq.encode())
        got_runs = [(int(iv[rec["n_first"] + q]["start"]), int(iv[rec["n_first"] + q]["end"]))
                    for q in range(rec["n_count"])]
        assert got_runs == runs
        want = [("ACGT".index(b.upper()) if b.upper() in "ACGT" else 0) for b in seq]
        assert list(codes[rec["base"]:rec["base"] + len(seq)]) == want


@pytest.mark.parametrize("mutate,msg", [
    (lambda b: b"PAIDXfmX" + b[8:], "bad magic"),
    (lambda b: b + b"\0" * 8, "trailing bytes after positions table"),
    (lambda b: b[:-3], "unexpected end of file"),
])
def test_rejects_like_the_reference(mutate, msg):
    with pytest.raises(S.PaidxError) as ei:
        S.paidx_scan(mutate(encode(SEQS, **TABLES)))
    assert str(ei.value) == msg and ei.value.code == -10


def test_version_and_table_checks():
    with pytest.raises(S.PaidxError) as ei:
        S.paidx_scan(encode(SEQS, version=2))
    assert ei.value.code == -11
    bad = dict(TABLES, kmers=[3, 3, 40])
    with pytest.raises(S.PaidxError, match="kmers not strictly ascending"):
        S.paidx_scan(encode(SEQS, **bad))
    bad = dict(TABLES, counts=[2, 1, 9])
    with pytest.raises(S.PaidxError, match="offset\\+count exceeds positions table"):
        S.paidx_scan(encode(SEQS, **bad))


def test_packed_len_tail_bits_and_pad():
    raw = bytearray(encode([("c", "ACG")]))
    # header 60 + counts 16; contig: name_len(4) name(1) seq_len(4) packed_len(4) packed(1)
    off_seq = 76 + 4 + 1
    bad = raw[:]
    bad[off_seq + 4:off_seq + 8] = struct.pack("<I", 2)
    with pytest.raises(S.PaidxError, match=r"packed_len != ceil\(seq_len/4\)"):
        S.paidx_scan(bytes(bad))
    bad = raw[:]
    bad[off_seq + 8] |= 0x01  # a bit of the unused fourth base
    with pytest.raises(S.PaidxError, match="non-zero tail bits in packed contig"):
        S.paidx_scan(bytes(bad))
    end_contigs = off_seq + 8 + 1 + 4
    bad = raw[:]
    bad[end_contigs] = 7  # first pad1 byte
    with pytest.raises(S.PaidxError, match="pad1 not zero"):
        S.paidx_scan(bytes(bad))
