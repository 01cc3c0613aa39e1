"""Host mirror of the splice-rescue flank DP of crates/map/src/split.rs over
the GB300 kernels, plus the resident genome it reads windows from.

* ``Genome``            -- the reference's ``Reference`` (fasta.rs:62-75):
                           2-bit contigs + N intervals, resident in HBM.
* ``retry_tail_start``  -- split.rs:150-223 (same arguments and result).
* ``channel_a_batch``   -- channel A (split.rs:468-570) over many reads, each
                           with its library candidates, + build_rescue_ext.
* ``score_tail_win``    -- splice.rs:667-684; ``tail_gate`` splice.rs:705-708.
* ``align_spliced``     -- splice.rs:617-664 on given exon slices: the DP on
                           the device-gathered pseudo-reference, stitch_cigar
                           (:435-493) and genomic_start (:414-424).
* ``paidx_contigs``     -- the contigs of a paidx v1 index (index_io.rs),
                           validated as the reference's loader does;
                           ``Genome.from_paidx`` makes them resident.
Every DP runs on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from . import batch as B
from .extend import (ExtendBuffer, ExtendParams, Extension, _b, _default_buffer,
                     decode_cigar)

SIG_GTAG, SIG_GCAG, SIG_ATAC, SIG_NONCANONICAL = 0, 1, 2, 3

CONTIG_DTYPE = np.dtype([("base", "<u8"), ("len", "<u4"), ("n_first", "<u4"),
                         ("n_count", "<u4"), ("pad", "<u4")])
SPLICE_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("tail_start", "<u4"),
                              ("contig", "<u4"), ("minus", "<i4"), ("cand_first", "<u4"),
                              ("cand_count", "<u4"), ("n_first", "<u4"), ("n_read", "<u4")])
SPLICE_CAND_DTYPE = np.dtype([("contig", "<u4"), ("start", "<u4"), ("end", "<u4"),
                              ("minus_strand", "<i4"), ("support", "<u4")])
SPLICE_RES_DTYPE = np.dtype([("found", "<i4"), ("cand", "<i4"), ("dro", "<u4"), ("pos", "<u4"),
                             ("score", "<i4"), ("signal", "<i4"), ("n_ops", "<u4"),
                             ("status", "<i4")])


@dataclass
class SpliceParams:
    """splice.rs:21-53 SpliceParams::default()."""
    min_intron: int = 20
    max_intron: int = 1_000_000
    gt_ag_bonus: int = 4
    gc_ag_bonus: int = 2
    at_ac_bonus: int = 1
    noncanonical_penalty: int = 8
    known_bonus: int = 6
    refine_radius: int = 12

    def _c(self):
        return N.SpliceParamsC(self.min_intron, self.max_intron, self.gt_ag_bonus,
                               self.gc_ag_bonus, self.at_ac_bonus, self.noncanonical_penalty,
                               self.known_bonus, self.refine_radius)


@dataclass
class Junction:
    """gtf.rs:23-32."""
    contig: int
    start: int
    end: int
    minus_strand: bool = False


@dataclass
class RetryOutcome:
    """split.rs:120-132."""
    dro: int
    left_win_lo: int
    left: Extension
    right: Extension
    total: int


class Genome:
    """A resident 2-bit genome: contigs packed MSB-first with their N runs."""

    def __init__(self, arena: np.ndarray, contigs: np.ndarray, n_iv: Optional[np.ndarray] = None,
                 buf: Optional[ExtendBuffer] = None):
        self.buf = buf or _default_buffer()
        self.arena = np.ascontiguousarray(arena, np.uint8)
        self.contigs = np.ascontiguousarray(contigs, CONTIG_DTYPE)
        self.n_iv = (np.zeros(0, B.NIV_DTYPE) if n_iv is None
                     else np.ascontiguousarray(n_iv, B.NIV_DTYPE))
        g = C.c_void_p()
        rc = N.lib().esp_genome_create(self.buf.handle, self.arena.ctypes.data, len(self.arena),
                                       self.contigs.ctypes.data, len(self.contigs),
                                       self.n_iv.ctypes.data if len(self.n_iv) else None,
                                       len(self.n_iv), C.byref(g))
        self.buf.check(rc)
        self._g = g

    @classmethod
    def from_sequences(cls, seqs: Sequence, buf: Optional[ExtendBuffer] = None) -> "Genome":
        """Contigs from ASCII sequences (non-ACGT -> N intervals)."""
        codes, contigs, ivs = [], np.zeros(len(seqs), CONTIG_DTYPE), []
        base = 0
        for c, s in enumerate(seqs):
            s = _b(s)
            arr = B._CODE[np.frombuffer(s, np.uint8)] if len(s) else np.zeros(0, np.uint8)
            isn = arr == 4
            runs = []
            k = 0
            while k < len(arr):
                if isn[k]:
                    e = k
                    while e < len(arr) and isn[e]:
                        e += 1
                    runs.append((k, e))
                    k = e
                else:
                    k += 1
            contigs[c] = (base, len(s), len(ivs), len(runs), 0)
            ivs.extend(runs)
            pad = (-len(arr)) % 4
            codes.append(np.concatenate([arr, np.zeros(pad, np.uint8)]))
            base += len(arr) + pad
        allc = np.concatenate(codes) if codes else np.zeros(0, np.uint8)
        n_iv = np.array(ivs, dtype=np.uint32).reshape(-1, 2)
        iv = np.zeros(len(n_iv), B.NIV_DTYPE)
        if len(n_iv):
            iv["start"], iv["end"] = n_iv[:, 0], n_iv[:, 1]
        return cls(B.pack_codes(allc), contigs, iv, buf)

    @classmethod
    def from_paidx(cls, data, buf: Optional[ExtendBuffer] = None) -> "Genome":
        """The contigs of a paidx v1 index (bytes or a path), resident."""
        arena, contigs, iv, _names, _info = paidx_contigs(data)
        return cls(arena, contigs, iv, buf)

    @property
    def handle(self):
        return self._g

    def close(self):
        if getattr(self, "_g", None):
            N.lib().esp_genome_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SPLICED_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("contig", "<u4"),
                               ("exon_first", "<u4"), ("exon_count", "<u4"),
                               ("n_first", "<u4"), ("n_read", "<u4")])
EXON_DTYPE = np.dtype([("start", "<u4"), ("end", "<u4")])
SPLICED_RES_DTYPE = np.dtype([("ext", B.EXT_DTYPE), ("genomic_start", "<u4"), ("n_ops", "<u4"),
                              ("status", "<i4"), ("pad", "<u4")])


def align_spliced_batch(genome: Genome, reads: Sequence, contigs: Sequence[int],
                        exon_lists: Sequence[Sequence[Tuple[int, int]]],
                        params: ExtendParams = ExtendParams(), cigar_stride: int = 64,
                        buf: Optional[ExtendBuffer] = None):
    """align_spliced for many reads, each with its contig and exon slices
    [(start, end)]: (SPLICED_RES_DTYPE records, extension CIGARs, stitched
    CIGARs), the CIGARs as (n, cigar_stride) u32 arrays."""
    buf = buf or _default_buffer()
    n = len(reads)
    reads = [_b(r) for r in reads]
    arena, pairs, n_iv = B.pack_ascii_pairs(reads, [b""] * n, [0] * n, [-1] * n)
    R = np.zeros(n, SPLICED_READ_DTYPE)
    ex = []
    for k in range(n):
        R[k] = (pairs["read_pos"][k], pairs["read_len"][k], contigs[k], len(ex),
                len(exon_lists[k]), pairs["n_first"][k], pairs["n_read"][k])
        ex.extend(exon_lists[k])
    E = np.array(ex, np.uint32).reshape(-1, 2).view(EXON_DTYPE).reshape(-1) if ex else \
        np.zeros(0, EXON_DTYPE)
    E = np.ascontiguousarray(E)
    out = np.zeros(n, SPLICED_RES_DTYPE)
    ecig = np.zeros((max(1, n), cigar_stride), np.uint32)
    scig = np.zeros((max(1, n), cigar_stride), np.uint32)
    p = params._c()
    niv = np.ascontiguousarray(n_iv, B.NIV_DTYPE)
    rc = N.lib().esp_batch_spliced_host(buf.handle, genome.handle, R.ctypes.data, n,
                                        arena.ctypes.data, len(arena),
                                        niv.ctypes.data if len(niv) else None, len(niv),
                                        E.ctypes.data if len(E) else None, len(E), C.byref(p),
                                        out.ctypes.data, ecig.ctypes.data, scig.ctypes.data,
                                        cigar_stride)
    buf.check(rc)
    return out, ecig[:n], scig[:n]


def align_spliced(genome: Genome, read, contig: int, exons: Sequence[Tuple[int, int]],
                  params: ExtendParams = ExtendParams(), buf: Optional[ExtendBuffer] = None):
    """One read: (Extension against the pseudo-reference, stitched CIGAR as
    [(op, len)], genomic start)."""
    stride = 2 * (len(_b(read)) + sum(e - s for s, e in exons)) + 2 * len(exons) + 8
    out, ecig, scig = align_spliced_batch(genome, [read], [contig], [exons], params, stride, buf)
    o = out[0]
    if o["status"] != 0:
        raise N.EspError(int(o["status"]), "align_spliced failed")
    x = o["ext"]
    ext = Extension(int(x["read_start"]), int(x["read_end"]), int(x["ref_start"]),
                    decode_cigar(ecig[0][:int(x["n_ops"])]), int(x["score"]))
    return ext, decode_cigar(scig[0][:int(o["n_ops"])]), int(o["genomic_start"])


class PaidxError(ValueError):
    """A malformed (ESP_EFORMAT) or unsupported (ESP_EVERSION) paidx file;
    the message is the reference loader's."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def _paidx_bytes(data) -> bytes:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return bytes(data)
    with open(data, "rb") as f:
        return f.read()


def paidx_scan(data) -> "N.PaidxInfoC":
    """Validate a paidx v1 file (index_io.rs:237-354 decode_parts) and size
    its contents; raises PaidxError with the reference's message."""
    raw = _paidx_bytes(data)
    info = N.PaidxInfoC()
    msg = C.create_string_buffer(256)
    rc = N.lib().esp_paidx_scan(raw, len(raw), C.byref(info), msg, 256)
    if rc != 0:
        raise PaidxError(rc, msg.value.decode())
    return info


def paidx_contigs(data):
    """(arena, contigs, n_intervals, names, info) of a paidx v1 file, laid
    out as a resident genome (each contig byte-aligned in the arena)."""
    raw = _paidx_bytes(data)
    info = paidx_scan(raw)
    arena = np.zeros(max(1, info.arena_bytes), np.uint8)
    contigs = np.zeros(info.contig_count, CONTIG_DTYPE)
    iv = np.zeros(max(1, info.n_iv_count), B.NIV_DTYPE)
    names = C.create_string_buffer(max(1, info.names_bytes))
    rc = N.lib().esp_paidx_contigs(raw, len(raw), arena.ctypes.data, len(arena),
                                   contigs.ctypes.data if len(contigs) else None, len(contigs),
                                   iv.ctypes.data, len(iv), names, len(names))
    if rc != 0:
        raise PaidxError(rc, "esp_paidx_contigs failed")
    nm = names.raw[:info.names_bytes].split(b"\0")[:info.contig_count]
    return (arena[:info.arena_bytes], contigs, iv[:info.n_iv_count],
            [x.decode("utf-8", "replace") for x in nm], info)


def score_tail_win(tail, ref_window, params: ExtendParams = ExtendParams(),
                   buf: Optional[ExtendBuffer] = None) -> Extension:
    """splice.rs:667-684: extend_hint of a tail along the direct diagonal."""
    buf = buf or _default_buffer()
    tail, ref_window = _b(tail), _b(ref_window)
    p = params._c()
    cap = 2 * (len(tail) + len(ref_window)) + 8
    ops = (C.c_uint32 * cap)()
    out = N.ExtensionC()
    buf.check(N.lib().esp_score_tail_win(buf.handle, tail, len(tail), ref_window,
                                         len(ref_window), C.byref(p), C.byref(out), ops, cap))
    return Extension(out.read_start, out.read_end, out.ref_start, decode_cigar(ops[:out.n_ops]),
                     out.score)


def tail_gate(ext: Extension, tail_len: int) -> bool:
    """splice.rs:705-708: aligned >= 4/5 of the tail and a positive score."""
    aligned = max(ext.read_end - ext.read_start, 0)
    return aligned * 5 >= tail_len * 4 and ext.score > 0


def retry_tail_start(genome: Genome, read, tail_start: int, j: Junction, signal: int,
                     support: int, params: SpliceParams = SpliceParams(),
                     extend_params: ExtendParams = ExtendParams(),
                     buf: Optional[ExtendBuffer] = None) -> Optional[RetryOutcome]:
    """split.rs:150-223 on the GPU."""
    buf = buf or genome.buf
    read = _b(read)
    cap = 2 * len(read) + 16
    lc, rc_ = (C.c_uint32 * cap)(), (C.c_uint32 * cap)()
    out = N.RetryOutcomeC()
    jc = N.JunctionC(j.contig, j.start, j.end, int(j.minus_strand))
    sp, p = params._c(), extend_params._c()
    rc = N.lib().esp_retry_tail_start(buf.handle, genome.handle, read, len(read), tail_start,
                                      C.byref(jc), signal, support, C.byref(sp), C.byref(p),
                                      C.byref(out), lc, rc_, cap)
    buf.check(rc)
    if not out.found:
        return None
    le = Extension(out.left.read_start, out.left.read_end, out.left.ref_start,
                   decode_cigar(lc[:out.left.n_ops]), out.left.score)
    re = Extension(out.right.read_start, out.right.read_end, out.right.ref_start,
                   decode_cigar(rc_[:out.right.n_ops]), out.right.score)
    return RetryOutcome(out.dro, out.left_win_lo, le, re, out.total)


def channel_a_batch(genome: Genome, reads: np.ndarray, read_arena: np.ndarray,
                    cands: np.ndarray, read_n_iv: Optional[np.ndarray] = None,
                    params: SpliceParams = SpliceParams(),
                    extend_params: ExtendParams = ExtendParams(), cigar_stride: int = 64,
                    buf: Optional[ExtendBuffer] = None):
    """Channel A over a batch: returns (results, cigars, dp_cells)."""
    buf = buf or genome.buf
    reads = np.ascontiguousarray(reads, SPLICE_READ_DTYPE)
    cands = np.ascontiguousarray(cands, SPLICE_CAND_DTYPE)
    read_arena = np.ascontiguousarray(read_arena, np.uint8)
    iv = (np.zeros(0, B.NIV_DTYPE) if read_n_iv is None
          else np.ascontiguousarray(read_n_iv, B.NIV_DTYPE))
    out = np.zeros(len(reads), SPLICE_RES_DTYPE)
    cig = np.zeros(max(1, len(reads) * cigar_stride), np.uint32)
    sp, p = params._c(), extend_params._c()
    rc = N.lib().esp_batch_splice_host(buf.handle, genome.handle, reads.ctypes.data, len(reads),
                                       read_arena.ctypes.data, len(read_arena),
                                       iv.ctypes.data if len(iv) else None, len(iv),
                                       cands.ctypes.data, len(cands), C.byref(sp), C.byref(p),
                                       out.ctypes.data, cig.ctypes.data, cigar_stride)
    buf.check(rc)
    cells = int(N.lib().esp_last_cells(buf.handle))
    return out, cig[:len(reads) * cigar_stride].reshape(len(reads), cigar_stride), cells


# ---- intron-chain fast path (intron_chain.rs:392-538 from the best pair on) ----

FRAG_DTYPE = [("q_lo", "<u4"), ("q_hi", "<u4"), ("r_lo", "<u4"), ("r_hi", "<u4"),
              ("n_anchors", "<u4")]
INTRON_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("contig", "<u4"),
                              ("n_first", "<u4"), ("n_read", "<u4"), ("minus", "<i4"),
                              ("intron_start", "<u4"), ("intron_end", "<u4"),
                              ("left", FRAG_DTYPE), ("right", FRAG_DTYPE), ("pad", "<u4")])
LIB_JUNCTION_DTYPE = np.dtype([("contig", "<u4"), ("start", "<u4"), ("end", "<u4"),
                               ("minus_strand", "<i4"), ("count", "<u4")])
INTRON_RES_DTYPE = np.dtype([("found", "<i4"), ("stage", "<i4"), ("donor_end", "<u4"),
                             ("acceptor_start", "<u4"), ("verify_donor", "<i4"),
                             ("verify_acceptor", "<i4"), ("j_contig", "<u4"), ("j_start", "<u4"),
                             ("j_end", "<u4"), ("j_minus", "<i4"), ("signal", "<i4"),
                             ("support", "<u4"), ("left_start", "<u4"), ("right_end", "<u4"),
                             ("ext", B.EXT_DTYPE), ("genomic_start", "<u4"), ("n_ops", "<u4"),
                             ("status", "<i4")])
assert INTRON_READ_DTYPE.itemsize == 80 and INTRON_RES_DTYPE.itemsize == 100
IC_STAGES = ("found", "empty", "anchors", "intron", "verify", "junction", "bounds", "result")


@dataclass
class IntronParams:
    """intron_chain.rs:21-41 IntronParams::default()."""
    min_frag_cov: int = 15
    refine_window: int = 30
    refine_pattern_len: int = 50
    intron_max: int = 105_000


def intron_chain_batch(genome: Genome, reads: np.ndarray, read_arena: np.ndarray,
                       junction_lib: np.ndarray, read_n_iv: Optional[np.ndarray] = None,
                       params: IntronParams = IntronParams(),
                       extend_params: ExtendParams = ExtendParams(), cigar_stride: int = 64,
                       buf: Optional[ExtendBuffer] = None):
    """try_intron_chain_placement over a batch of reads with their best
    fragment pairs: (results, extension CIGARs, stitched CIGARs)."""
    buf = buf or genome.buf
    reads = np.ascontiguousarray(reads, INTRON_READ_DTYPE)
    read_arena = np.ascontiguousarray(read_arena, np.uint8)
    lib = np.ascontiguousarray(junction_lib, LIB_JUNCTION_DTYPE)
    iv = (np.zeros(0, B.NIV_DTYPE) if read_n_iv is None
          else np.ascontiguousarray(read_n_iv, B.NIV_DTYPE))
    n = len(reads)
    out = np.zeros(n, INTRON_RES_DTYPE)
    ec = np.zeros(max(1, n * cigar_stride), np.uint32)
    sc = np.zeros(max(1, n * cigar_stride), np.uint32)
    ip = (C.c_uint32 * 4)(params.min_frag_cov, params.refine_window, params.refine_pattern_len,
                          params.intron_max)
    p = extend_params._c()
    L = N.lib()
    fn = L.esp_batch_intron_chain_host
    fn.argtypes = [C.c_void_p] * 3 + [C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                      C.c_void_p, C.c_uint64, C.c_void_p,
                                      C.POINTER(N.ExtendParamsC), C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_uint32]
    rc = fn(buf.handle, genome.handle, reads.ctypes.data, n, read_arena.ctypes.data,
            len(read_arena), iv.ctypes.data if len(iv) else None, len(iv),
            lib.ctypes.data if len(lib) else None, len(lib), ip, C.byref(p), out.ctypes.data,
            ec.ctypes.data, sc.ctypes.data, cigar_stride)
    buf.check(rc)
    return (out, ec[:n * cigar_stride].reshape(n, cigar_stride),
            sc[:n * cigar_stride].reshape(n, cigar_stride))
