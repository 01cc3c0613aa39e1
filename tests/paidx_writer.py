"""Test fixture writer for the paidx v1 byte layout (crates/map/src/index_io.rs:1-16
and its encode, :44-110): header, contigs (2-bit MSB-first packed with N
intervals, fasta.rs:1-5), pad1, k-mer tables, pad2, positions.  It restates
the published layout so the reader can be checked on files built here."""
import struct

CODES = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}


def pack_contig(seq: bytes):
    """(packed bytes, N intervals) as fasta.rs stores a contig: non-ACGT bases
    are N runs and pack as 0; tail bits of the last byte stay zero."""
    packed = bytearray((len(seq) + 3) // 4)
    runs, k = [], 0
    for i, b in enumerate(seq):
        code = CODES.get(b & ~0x20 if 97 <= b <= 122 else b)
        if code is None:
            if runs and runs[-1][1] == i:
                runs[-1][1] = i + 1
            else:
                runs.append([i, i + 1])
            code = 0
        packed[i // 4] |= code << (6 - 2 * (i % 4))
    return bytes(packed), [tuple(r) for r in runs]


def encode(contigs, k=5, w=2, freq_cutoff=0, kmers=(), offsets=(), counts=(), positions=(),
           sha=b"\x11" * 32, version=1):
    """contigs: list of (name, ASCII sequence)."""
    body = bytearray()
    for name, seq in contigs:
        nb = name.encode()
        packed, runs = pack_contig(seq if isinstance(seq, bytes) else seq.encode())
        body += struct.pack("<I", len(nb)) + nb
        body += struct.pack("<II", len(seq), len(packed)) + packed
        body += struct.pack("<I", len(runs))
        for s, e in runs:
            body += struct.pack("<II", s, e)
    head = b"PAIDXfmt" + struct.pack("<IIIII", version, k, w, freq_cutoff, len(contigs))
    head += struct.pack("<QQ", len(kmers), len(positions)) + sha
    out = bytearray(head) + body
    out += b"\0" * ((8 - len(out) % 8) % 8)  # pad1
    for v in kmers:
        out += struct.pack("<Q", v)
    for v in offsets:
        out += struct.pack("<Q", v)
    for v in counts:
        out += struct.pack("<I", v)
    out += b"\0" * ((8 - len(out) % 8) % 8)  # pad2
    for v in positions:
        out += struct.pack("<Q", v)
    return bytes(out)
