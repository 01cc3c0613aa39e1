"""The oracle's read-aware junction refinement (splice.rs:208-313
refine_junction_read; oracle/intron.c), pinned to the reference's own
boundary test (splice.rs:894-960,
read_boundary_competition_is_invariant_to_mate_orientation): a 500-base
xorshift genome with a GT..AG (or, for a minus-strand transcript, CT..AC)
intron at [120, 300), a competing donor just after the acceptor and a
mismatch at the read's last exon-1 base.  For both transcript strands, an
annotated or empty junction library, both read orientations and seed
boundaries shifted by 1 and 2, the refinement must pick the planted
junction with its strand, a GT-AG signal and the library support."""
import ctypes as C

import oracle as O

M64 = (1 << 64) - 1


def _genome():
    # the reference test's generator: xorshift64 (13, 7, 17) from 0x243f6a88
    state = 0x243F6A88
    out = bytearray()
    for _ in range(500):
        state ^= (state << 13) & M64
        state ^= state >> 7
        state ^= (state << 17) & M64
        out.append(b"ACGT"[state & 3])
    return out


def _refine(contig, read, naive_start, naive_end, q_a, q_b, minus, lib):
    L = O.lib()
    fn = L.orc_refine_junction_read
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32,
                   C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.c_uint64, C.c_void_p,
                   C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_uint32)]
    entries = (O._LibEntry * max(1, len(lib)))(*[O._LibEntry(*e) for e in lib])
    sp = O.splice_params_default()
    out = O._Junction()
    sig, sup = C.c_int(), C.c_uint32()
    have = fn(C.addressof(contig.c), 0, bytes(read), len(read), naive_start, naive_end, q_a,
              q_b, int(minus), C.addressof(entries), len(lib), C.addressof(sp),
              C.addressof(out), C.byref(sig), C.byref(sup))
    return have, (out.start, out.end, bool(out.minus_strand)), sig.value, sup.value


def test_read_boundary_competition_is_invariant_to_mate_orientation():
    genome = _genome()
    checked = 0
    for transcript_minus in (False, True):
        donor, acceptor = (b"CT", b"AC") if transcript_minus else (b"GT", b"AG")
        genome[120:122] = donor
        genome[298:300] = acceptor
        genome[300:302] = donor
        genome[119] = ord("T")
        query = bytearray(genome[60:120])
        query[59] = ord("C")
        query += genome[300:379]
        contig = O.Contig(bytes(genome))
        for annotated in (False, True):
            lib = [(0, 120, 300, int(transcript_minus), 1)] if annotated else []
            for read_minus in (False, True):
                for shift in (1, 2):
                    have, junction, signal, support = _refine(
                        contig, query, 120 + shift, 300 + shift, 60 + shift, 60 + shift,
                        read_minus, lib)
                    assert have, (transcript_minus, annotated, read_minus, shift)
                    assert junction == (120, 300, transcript_minus), (
                        transcript_minus, annotated, read_minus, shift, junction)
                    assert signal == O.SIG_GTAG
                    assert support == int(annotated)
                    checked += 1
    assert checked == 16
