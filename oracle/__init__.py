"""CPU oracle for the ESPERANTO read-alignment inner loop (TEST INFRASTRUCTURE).

This package wraps the C restatement in this directory (extend.c, myers.c,
split.c, batch.c) with ctypes.  Only the test suite, the smoke check and the
CPU-baseline leg of the benchmark may load it; the product package never
imports it.  Each C function cites the reference Rust file:line it restates.

Parity pins: the reference (a Rust workspace) cannot be built here, so the
restatement is pinned against the literal known answers of the reference's
own unit tests (tests/golden/known_answers.json, tests/test_oracle_*.py), a
brute-force edit-distance DP for both Myers formulations, and agreement of
the i16 and i32 kernel flavours on the reference's seeded sweeps.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libesp_oracle.so")
SOURCES = ["extend.c", "myers.c", "split.c", "batch.c", "rescore.c", "spliced.c", "intron.c"]

OP_M, OP_I, OP_D, OP_N, OP_S = 0, 1, 2, 3, 4
OP_CHARS = "MIDNS"
EDIT_OFF, EDIT_AG, EDIT_TC = 0, 1, 2


SYNTH_SRC = os.path.join(os.path.dirname(HERE), "workloads", "synth.cpp")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc into oracle/_build (portable C, -O3, the
    optimisation level of the reference's own release builds).  The library
    also carries a g++ build of the seeded workload generators
    (workloads/synth.cpp), so that the benchmark's reference arm makes its
    inputs without loading any library of the GPU path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    inc = [os.path.join(os.path.dirname(HERE), "workloads"),
           os.path.join(os.path.dirname(HERE), "include")]
    deps = ([os.path.join(HERE, s) for s in SOURCES] + [SYNTH_SRC, os.path.join(HERE, "esp_oracle.h"),
            os.path.abspath(__file__)] + [os.path.join(d, h) for d, h in
                                          ((inc[0], "esp_workloads.h"), (inc[1], "esperanto_gb300.h"))])
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_m for s in deps):
            return LIB_PATH
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, src + ".o")
        subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-pthread", "-Wall", "-c",
                        os.path.join(HERE, src), "-o", obj], check=True)
        objs.append(obj)
    obj = os.path.join(BUILD_DIR, "synth.cpp.o")
    subprocess.run(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-I", inc[0], "-I", inc[1],
                    "-c", SYNTH_SRC, "-o", obj], check=True)
    objs.append(obj)
    subprocess.run(["g++", "-shared", "-pthread", "-o", LIB_PATH + ".tmp"] + objs + ["-lm"],
                   check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class _Params(C.Structure):
    _fields_ = [("match_score", C.c_int32), ("mismatch", C.c_int32), ("gap_open", C.c_int32),
                ("gap_ext", C.c_int32), ("edit_dir", C.c_int32)]


class _Ext(C.Structure):
    _fields_ = [("read_start", C.c_uint32), ("read_end", C.c_uint32), ("ref_start", C.c_uint32),
                ("score", C.c_int32), ("n_ops", C.c_uint32), ("cap", C.c_uint32),
                ("ops", C.POINTER(C.c_uint32))]


class _Touch(C.Structure):
    _fields_ = [("touched", C.c_int32), ("row", C.c_int64), ("left", C.c_int32),
                ("clamped", C.c_int32)]


class _Contig(C.Structure):
    _fields_ = [("len", C.c_uint32), ("packed", C.c_void_p), ("n_iv", C.c_void_p),
                ("n_iv_count", C.c_uint32)]


class _SpliceParams(C.Structure):
    _fields_ = [("min_intron", C.c_uint32), ("max_intron", C.c_uint32),
                ("gt_ag_bonus", C.c_int32), ("gc_ag_bonus", C.c_int32),
                ("at_ac_bonus", C.c_int32), ("noncanonical_penalty", C.c_int32),
                ("known_bonus", C.c_int32), ("refine_radius", C.c_uint32)]


class _Junction(C.Structure):
    _fields_ = [("start", C.c_uint32), ("end", C.c_uint32), ("minus_strand", C.c_int32)]


class _Retry(C.Structure):
    _fields_ = [("found", C.c_int32), ("dro", C.c_uint32), ("left_win_lo", C.c_uint32),
                ("total", C.c_int32), ("left", _Ext), ("right", _Ext)]


class _Rescue(C.Structure):
    _fields_ = [("found", C.c_int32), ("cand", C.c_int32), ("dro", C.c_uint32),
                ("pos", C.c_uint32), ("score", C.c_int32), ("signal", C.c_int32),
                ("n_ops", C.c_uint32), ("cap", C.c_uint32), ("ops", C.POINTER(C.c_uint32))]


class _Pairs(C.Structure):
    _fields_ = [("seqs", C.c_void_p), ("read_off", C.c_void_p), ("read_len", C.c_void_p),
                ("win_off", C.c_void_p), ("win_len", C.c_void_p), ("offset", C.c_void_p),
                ("half", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()  # no-op when the library is newer than every source
        L = C.CDLL(LIB_PATH)
        u8p = C.c_char_p
        i64, i32 = C.c_int64, C.c_int32
        L.orc_run_band.argtypes = [u8p, i64, u8p, i64, C.POINTER(_Params), C.c_int, C.c_int,
                                   i64, i64, i64, i64, C.POINTER(_Ext), C.POINTER(_Touch)]
        L.orc_run_dispatch.argtypes = [u8p, i64, u8p, i64, C.POINTER(_Params), C.c_int, i64,
                                       i64, i64, i64, C.POINTER(_Ext), C.POINTER(_Touch)]
        L.orc_extend.argtypes = [u8p, i64, u8p, i64, C.POINTER(_Params), C.POINTER(_Ext)]
        for name in ("orc_extend_hint", "orc_extend_hint_i32"):
            getattr(L, name).argtypes = [u8p, i64, u8p, i64, C.POINTER(_Params), i64,
                                         C.c_uint32, C.c_uint32, C.POINTER(_Ext),
                                         C.POINTER(C.c_int)]
        L.orc_band_cells.argtypes = [i64, i64, C.c_int, i64, i64]
        L.orc_band_cells.restype = i64
        L.orc_i16_add.argtypes = [C.c_int16, C.c_int16]
        L.orc_i16_add.restype = C.c_int16
        for name in ("orc_myers_infix_best_end", "orc_myers_infix_best_start",
                     "orc_myers_long_infix_best_end", "orc_myers_long_infix_best_start",
                     "orc_ea_edit_dp"):
            getattr(L, name).argtypes = [u8p, i64, u8p, i64, C.POINTER(i32), C.POINTER(i64)]
        for name in ("orc_myers_infix", "orc_myers_long_infix"):
            getattr(L, name).argtypes = [u8p, i64, u8p, i64, C.POINTER(i32)]
        for name in ("orc_engine_infix", "orc_engine_global"):
            getattr(L, name).argtypes = [u8p, i64, u8p, i64, C.POINTER(C.c_uint32)]
        L.orc_splice_signal.argtypes = [u8p, u8p, C.c_int]
        L.orc_signal_score.argtypes = [C.c_int, C.POINTER(_SpliceParams)]
        L.orc_junction_signal.argtypes = [C.POINTER(_Contig), C.POINTER(_Junction)]
        L.orc_splice_params_default.argtypes = [C.POINTER(_SpliceParams)]
        L.orc_cigar_ref_end.argtypes = [C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32]
        L.orc_cigar_ref_end.restype = C.c_uint32
        L.orc_retry_tail_start.argtypes = [C.POINTER(_Contig), u8p, C.c_uint32, C.c_uint32,
                                           C.POINTER(_Junction), C.c_int, C.c_uint32,
                                           C.POINTER(_SpliceParams), C.POINTER(_Params),
                                           C.POINTER(_Retry)]
        L.orc_channel_a.argtypes = [C.POINTER(_Contig), u8p, C.c_uint32, C.c_uint32, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.POINTER(_SpliceParams), C.POINTER(_Params),
                                    C.POINTER(_Rescue)]
        L.orc_slice_ascii.argtypes = [C.POINTER(_Contig), C.c_uint32, C.c_uint32, C.c_void_p]
        L.orc_pack_2bit.argtypes = [u8p, i64, C.c_void_p]
        L.orc_batch_extend.argtypes = [C.POINTER(_Pairs), i64, C.POINTER(_Params), C.c_int,
                                       C.c_int] + [C.c_void_p] * 6 + [C.c_uint32, C.c_void_p]
        L.orc_batch_extend.restype = i64
        L.orc_batch_myers_best_end.argtypes = [C.c_void_p] * 5 + [i64, C.c_int, C.c_void_p,
                                                                   C.c_void_p]
        L.orc_batch_myers_best_end.restype = i64
        L.orc_batch_channel_a.argtypes = [C.c_void_p] * 13 + [i64, C.c_int, C.c_void_p,
                                                               C.c_void_p, C.c_void_p,
                                                               C.c_void_p]
        L.free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def synth_lib():
    """This library's build of the workload generators, bound like
    workloads.synth_lib() (pass it as ``lib=`` to the workloads generators)."""
    import workloads
    return workloads.bind_synth(lib())


def _libc_free(ptr):
    C.CDLL(None).free(C.cast(ptr, C.c_void_p))


@dataclass
class Params:
    """ExtendParams (crates/map/src/extend.rs:97-122)."""
    match_score: int = 2
    mismatch: int = -4
    gap_open: int = 4
    gap_ext: int = 2
    edit_dir: int = EDIT_OFF

    def c(self) -> _Params:
        return _Params(self.match_score, self.mismatch, self.gap_open, self.gap_ext,
                       self.edit_dir)


@dataclass
class Ext:
    read_start: int
    read_end: int
    ref_start: int
    score: int
    cigar: List[Tuple[str, int]] = field(default_factory=list)

    def key(self):
        return (self.score, self.read_start, self.read_end, self.ref_start, tuple(self.cigar))


@dataclass
class Touch:
    touched: bool
    row: int
    left: bool
    clamped: bool


class OracleError(RuntimeError):
    pass


def decode_ops(ops) -> List[Tuple[str, int]]:
    return [(OP_CHARS[o & 15], o >> 4) for o in ops]


def _b(s) -> bytes:
    return s.encode() if isinstance(s, str) else bytes(s)


def _call_ext(fn, *args, m: int, n: int):
    cap = 2 * (m + n) + 8
    buf = (C.c_uint32 * cap)()
    e = _Ext(0, 0, 0, 0, 0, cap, buf)
    rc = fn(*args, C.byref(e))
    if rc != 0:
        raise OracleError(f"oracle returned {rc}")
    return Ext(e.read_start, e.read_end, e.ref_start, e.score, decode_ops(buf[:e.n_ops]))


def run_band(read, win, params: Params = Params(), wide: bool = False,
             band: Optional[Tuple[int, int]] = None) -> Tuple[Ext, Touch]:
    """run_band<T> (extend.rs:606-851); band = (offset, half) or None."""
    read, win = _b(read), _b(win)
    p = params.c()
    t = _Touch()
    off, half = band if band is not None else (0, 0)
    cap = 2 * (len(read) + len(win)) + 8
    buf = (C.c_uint32 * cap)()
    e = _Ext(0, 0, 0, 0, 0, cap, buf)
    rc = lib().orc_run_band(read, len(read), win, len(win), C.byref(p), int(wide),
                            int(band is not None), off, 1, 1, half, C.byref(e), C.byref(t))
    if rc != 0:
        raise OracleError(f"orc_run_band returned {rc}")
    return (Ext(e.read_start, e.read_end, e.ref_start, e.score, decode_ops(buf[:e.n_ops])),
            Touch(bool(t.touched), t.row, bool(t.left), bool(t.clamped)))


def run_dispatch(read, win, params: Params = Params(),
                 band: Optional[Tuple[int, int]] = None) -> Tuple[Ext, Touch]:
    read, win = _b(read), _b(win)
    p = params.c()
    t = _Touch()
    off, half = band if band is not None else (0, 0)
    cap = 2 * (len(read) + len(win)) + 8
    buf = (C.c_uint32 * cap)()
    e = _Ext(0, 0, 0, 0, 0, cap, buf)
    rc = lib().orc_run_dispatch(read, len(read), win, len(win), C.byref(p),
                                int(band is not None), off, 1, 1, half, C.byref(e), C.byref(t))
    if rc != 0:
        raise OracleError(f"orc_run_dispatch returned {rc}")
    return (Ext(e.read_start, e.read_end, e.ref_start, e.score, decode_ops(buf[:e.n_ops])),
            Touch(bool(t.touched), t.row, bool(t.left), bool(t.clamped)))


def extend(read, win, params: Params = Params()) -> Ext:
    read, win = _b(read), _b(win)
    p = params.c()
    return _call_ext(lib().orc_extend, read, len(read), win, len(win), C.byref(p),
                     m=len(read), n=len(win))


def extend_hint(read, win, params: Params = Params(), offset: int = 0,
                with_escalation: bool = False, wide: bool = False):
    """extend_hint (extend.rs:392-428); wide = every attempt in the i32
    flavour of run_band (extend.rs:462-528)."""
    read, win = _b(read), _b(win)
    p = params.c()
    esc = C.c_int(0)
    cap = 2 * (len(read) + len(win)) + 8
    buf = (C.c_uint32 * cap)()
    e = _Ext(0, 0, 0, 0, 0, cap, buf)
    fn = lib().orc_extend_hint_i32 if wide else lib().orc_extend_hint
    rc = fn(read, len(read), win, len(win), C.byref(p), offset, 1, 1, C.byref(e), C.byref(esc))
    if rc != 0:
        raise OracleError(f"orc_extend_hint returned {rc}")
    ext = Ext(e.read_start, e.read_end, e.ref_start, e.score, decode_ops(buf[:e.n_ops]))
    return (ext, bool(esc.value)) if with_escalation else ext


def band_cells(m: int, n: int, band: Optional[Tuple[int, int]]) -> int:
    if band is None:
        return lib().orc_band_cells(m, n, 0, 0, 0)
    return lib().orc_band_cells(m, n, 1, band[0], band[1])


def i16_add(a: int, b: int) -> int:
    return lib().orc_i16_add(a, b)


def _myers2(fn, read, text):
    read, text = _b(read), _b(text)
    d, e = C.c_int32(), C.c_int64()
    rc = fn(read, len(read), text, len(text), C.byref(d), C.byref(e))
    if rc != 0:
        raise OracleError(f"myers oracle returned {rc}")
    return d.value, e.value


def myers_infix(read, text) -> int:
    read, text = _b(read), _b(text)
    d = C.c_int32()
    rc = lib().orc_myers_infix(read, len(read), text, len(text), C.byref(d))
    if rc != 0:
        raise OracleError(f"orc_myers_infix returned {rc}")
    return d.value


def myers_long_infix(read, text) -> int:
    read, text = _b(read), _b(text)
    d = C.c_int32()
    rc = lib().orc_myers_long_infix(read, len(read), text, len(text), C.byref(d))
    if rc != 0:
        raise OracleError(f"orc_myers_long_infix returned {rc}")
    return d.value


def myers_infix_best_end(read, text):
    return _myers2(lib().orc_myers_infix_best_end, read, text)


def myers_infix_best_start(read, text):
    return _myers2(lib().orc_myers_infix_best_start, read, text)


def myers_long_infix_best_end(read, text):
    return _myers2(lib().orc_myers_long_infix_best_end, read, text)


def myers_long_infix_best_start(read, text):
    return _myers2(lib().orc_myers_long_infix_best_start, read, text)


def ea_edit_dp(read, text):
    return _myers2(lib().orc_ea_edit_dp, read, text)


def engine_infix(read, text) -> int:
    read, text = _b(read), _b(text)
    d = C.c_uint32()
    rc = lib().orc_engine_infix(read, len(read), text, len(text), C.byref(d))
    if rc != 0:
        raise OracleError(f"orc_engine_infix returned {rc}")
    return d.value


def engine_global(read, text) -> int:
    read, text = _b(read), _b(text)
    d = C.c_uint32()
    rc = lib().orc_engine_global(read, len(read), text, len(text), C.byref(d))
    if rc != 0:
        raise OracleError(f"orc_engine_global returned {rc}")
    return d.value


# ---- reference storage / splice ----

def pack_2bit(seq) -> bytes:
    seq = _b(seq)
    out = (C.c_uint8 * ((len(seq) + 3) // 4))()
    lib().orc_pack_2bit(seq, len(seq), out)
    return bytes(out)


def n_intervals(seq) -> List[Tuple[int, int]]:
    """Merged half-open runs of non-ACGT bytes (the contig's N list)."""
    out: List[Tuple[int, int]] = []
    s = None
    for k, b in enumerate(_b(seq)):
        isn = chr(b) not in "ACGTacgt"
        if isn and s is None:
            s = k
        elif not isn and s is not None:
            out.append((s, k))
            s = None
    if s is not None:
        out.append((s, len(seq)))
    return out


class Contig:
    """A 2-bit packed contig with N intervals (crates/map/src/fasta.rs:62-135)."""

    def __init__(self, seq):
        seq = _b(seq)
        self.len = len(seq)
        self.packed = pack_2bit(seq)
        ivs = n_intervals(seq)
        self._pk = (C.c_uint8 * max(1, len(self.packed))).from_buffer_copy(
            self.packed or b"\0")
        flat = [v for iv in ivs for v in iv]
        self._iv = (C.c_uint32 * max(1, len(flat)))(*flat)
        self.n_iv = ivs
        self.c = _Contig(self.len, C.cast(self._pk, C.c_void_p), C.cast(self._iv, C.c_void_p),
                         len(ivs))

    def slice_ascii(self, start: int, end: int) -> bytes:
        out = (C.c_uint8 * max(1, end - start))()
        lib().orc_slice_ascii(C.byref(self.c), start, end, out)
        return bytes(out[: end - start])


SIG_GTAG, SIG_GCAG, SIG_ATAC, SIG_NONCANON = 0, 1, 2, 3


def splice_params_default() -> _SpliceParams:
    sp = _SpliceParams()
    lib().orc_splice_params_default(C.byref(sp))
    return sp


def splice_signal(donor, acceptor, minus: bool) -> int:
    return lib().orc_splice_signal(_b(donor), _b(acceptor), int(minus))


def junction_signal(contig: Contig, start: int, end: int, minus: bool) -> int:
    j = _Junction(start, end, int(minus))
    return lib().orc_junction_signal(C.byref(contig.c), C.byref(j))


def cigar_ref_end(pos: int, cigar: Sequence[Tuple[str, int]]) -> int:
    ops = [(n << 4) | OP_CHARS.index(c) for c, n in cigar]
    arr = (C.c_uint32 * max(1, len(ops)))(*ops)
    return lib().orc_cigar_ref_end(pos, arr, len(ops))


@dataclass
class Retry:
    dro: int
    left_win_lo: int
    total: int
    left: Ext
    right: Ext


def retry_tail_start(contig: Contig, read, tail_start: int, start: int, end: int,
                     minus: bool, signal: int, support: int,
                     params: Params = Params()) -> Optional[Retry]:
    """split.rs:150-223 retry_tail_start."""
    read = _b(read)
    sp = splice_params_default()
    p = params.c()
    j = _Junction(start, end, int(minus))
    o = _Retry()
    rc = lib().orc_retry_tail_start(C.byref(contig.c), read, len(read), tail_start,
                                    C.byref(j), signal, support, C.byref(sp), C.byref(p),
                                    C.byref(o))
    if rc != 0:
        raise OracleError(f"orc_retry_tail_start returned {rc}")
    if not o.found:
        return None
    le = Ext(o.left.read_start, o.left.read_end, o.left.ref_start, o.left.score,
             decode_ops(o.left.ops[: o.left.n_ops]))
    re = Ext(o.right.read_start, o.right.read_end, o.right.ref_start, o.right.score,
             decode_ops(o.right.ops[: o.right.n_ops]))
    _libc_free(o.left.ops)
    _libc_free(o.right.ops)
    return Retry(o.dro, o.left_win_lo, o.total, le, re)


@dataclass
class Rescue:
    cand: int
    dro: int
    pos: int
    score: int
    signal: int
    cigar: List[Tuple[str, int]]


def channel_a(contig: Contig, read, tail_start: int, minus: bool,
              cands: Sequence[Tuple[int, int, bool]], support: Sequence[int],
              params: Params = Params()) -> Optional[Rescue]:
    """split.rs:468-570 channel A over caller-supplied candidates."""
    read = _b(read)
    sp = splice_params_default()
    p = params.c()
    js = (_Junction * max(1, len(cands)))(*[_Junction(s, e, int(mi)) for s, e, mi in cands])
    sup = (C.c_uint32 * max(1, len(support)))(*support)
    cap = 4 * len(read) + 16
    buf = (C.c_uint32 * cap)()
    o = _Rescue(0, 0, 0, 0, 0, 0, 0, cap, buf)
    rc = lib().orc_channel_a(C.byref(contig.c), read, len(read), tail_start, int(minus),
                             C.cast(js, C.c_void_p), C.cast(sup, C.c_void_p), len(cands),
                             C.byref(sp), C.byref(p), C.byref(o))
    if rc != 0:
        raise OracleError(f"orc_channel_a returned {rc}")
    if not o.found:
        return None
    return Rescue(o.cand, o.dro, o.pos, o.score, o.signal, decode_ops(buf[: o.n_ops]))


# ---- batch drivers (CPU baseline) ----

def batch_extend(seqs, read_off, read_len, win_off, win_len, offset, half, params: Params,
                 mode: int, threads: int, ops_stride: int = 0):
    """Run the oracle over a batch with `threads` workers.  Arrays are numpy.
    mode 0 = run_dispatch with each pair's band (half < 0: full matrix),
    mode 1 = extend_hint with each pair's offset.  Returns (cells, outputs)."""
    import numpy as np
    n = len(read_len)
    keep = [np.ascontiguousarray(a) for a in (seqs, read_off.astype(np.uint64),
                                               read_len.astype(np.uint32),
                                               win_off.astype(np.uint64),
                                               win_len.astype(np.uint32),
                                               offset.astype(np.int64), half.astype(np.int32))]
    pr = _Pairs(*[a.ctypes.data for a in keep])
    score = np.zeros(n, np.int32)
    rs = np.zeros(n, np.uint32)
    re = np.zeros(n, np.uint32)
    fs = np.zeros(n, np.uint32)
    nops = np.zeros(n, np.uint32)
    touched = np.zeros(n, np.int32)
    ops = np.zeros(max(1, n * ops_stride), np.uint32) if ops_stride else None
    p = params.c()
    cells = lib().orc_batch_extend(C.byref(pr), n, C.byref(p), mode, threads,
                                   score.ctypes.data, rs.ctypes.data, re.ctypes.data,
                                   fs.ctypes.data, nops.ctypes.data,
                                   ops.ctypes.data if ops is not None else None, ops_stride,
                                   touched.ctypes.data)
    if cells < 0:
        raise OracleError(f"orc_batch_extend returned {cells}")
    out = dict(score=score, read_start=rs, read_end=re, ref_start=fs, n_ops=nops,
               touched=touched)
    if ops is not None:
        out["ops"] = ops.reshape(n, ops_stride)
    return int(cells), out


def batch_myers_best_end(seqs, read_off, read_len, text_off, text_len, threads: int):
    import numpy as np
    n = len(read_len)
    keep = [np.ascontiguousarray(a) for a in (seqs, read_off.astype(np.uint64),
                                               read_len.astype(np.uint32),
                                               text_off.astype(np.uint64),
                                               text_len.astype(np.uint32))]
    dist = np.zeros(n, np.int32)
    end = np.zeros(n, np.int64)
    cells = lib().orc_batch_myers_best_end(*[a.ctypes.data for a in keep], n, threads,
                                           dist.ctypes.data, end.ctypes.data)
    if cells < 0:
        raise OracleError(f"orc_batch_myers_best_end returned {cells}")
    return int(cells), dist, end


class _CaDetail(C.Structure):
    _fields_ = [("cand", C.c_void_p), ("dro", C.c_void_p), ("pos", C.c_void_p),
                ("signal", C.c_void_p), ("n_ops", C.c_void_p), ("ops", C.c_void_p),
                ("ops_stride", C.c_uint32)]


def batch_channel_a(garena, contigs, read_ascii, read_off, reads, cands, threads: int,
                    ops_stride: int = 0):
    """Channel A per read with `threads` workers (plus strand, defaults).
    Returns (found, score, dp_cells), or with ops_stride > 0
    (found, score, dp_cells, detail) where detail holds per read the winning
    candidate (-1 when none), dro, pos, signal, n_ops and the spliced CIGAR
    (first ops_stride ops)."""
    import numpy as np
    n = len(reads)
    keep = [np.ascontiguousarray(a) for a in (
        garena, contigs["base"].astype(np.uint64), contigs["len"].astype(np.uint32), read_ascii,
        read_off.astype(np.uint64), reads["read_len"].astype(np.uint32),
        reads["tail_start"].astype(np.uint32), reads["contig"].astype(np.uint32),
        reads["cand_first"].astype(np.uint32), reads["cand_count"].astype(np.uint32),
        cands["start"].astype(np.uint32), cands["end"].astype(np.uint32),
        cands["support"].astype(np.uint32))]
    found = np.zeros(n, np.int32)
    score = np.zeros(n, np.int32)
    cells = C.c_int64()
    det = None
    if ops_stride:
        det = dict(cand=np.zeros(n, np.int32), dro=np.zeros(n, np.uint32),
                   pos=np.zeros(n, np.uint32), signal=np.zeros(n, np.int32),
                   n_ops=np.zeros(n, np.uint32), ops=np.zeros((n, ops_stride), np.uint32))
        d = _CaDetail(*[det[k].ctypes.data for k in ("cand", "dro", "pos", "signal", "n_ops",
                                                      "ops")], ops_stride)
    rc = lib().orc_batch_channel_a(*[a.ctypes.data for a in keep], n, threads,
                                   found.ctypes.data, score.ctypes.data, C.byref(cells),
                                   C.byref(d) if det is not None else None)
    if rc != 0:
        raise OracleError(f"orc_batch_channel_a returned {rc}")
    if det is not None:
        return found, score, cells.value, det
    return found, score, cells.value


class _Strict(C.Structure):
    _fields_ = [("score", C.c_int32), ("aligned", C.c_uint32), ("matches", C.c_uint32),
                ("mm", C.c_uint32), ("ea_ag", C.c_uint32), ("ea_tc", C.c_uint32),
                ("ins", C.c_uint32), ("del_", C.c_uint32), ("clipped", C.c_uint32),
                ("n_splice", C.c_uint32), ("splice_score", C.c_int32)]


STRICT_FIELDS = ("score", "aligned", "matches", "mm", "ea_ag", "ea_tc", "ins", "del_", "clipped",
                 "n_splice", "splice_score")


def intron_length_penalty(n: int) -> int:
    """splice.rs:119-121 (host libm log10)."""
    f = lib().orc_intron_length_penalty
    f.restype = C.c_int32
    f.argtypes = [C.c_uint32]
    return f(n)


def rescore(contig: "Contig", contig_id: int, pos: int, query, ops, junction_lib=(),
            params: Params = Params(), edit_dir: int = 0):
    """align.rs:1060-1165 rescore_with: the StrictScore of a placement as a
    tuple in STRICT_FIELDS order.  ops: u32 (len << 4 | op), M I D N S = 0..4;
    junction_lib: (contig, start, end) sorted."""
    q = _b(query)
    arr = (C.c_uint32 * max(1, len(ops)))(*ops)
    flat = [v for j in junction_lib for v in j]
    jl = (C.c_uint32 * max(1, len(flat)))(*flat)
    s = _Strict()
    f = lib().orc_rescore
    f.restype = None
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_char_p, C.c_uint32, C.c_void_p,
                  C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int, C.c_void_p]
    f(C.byref(contig.c), contig_id, pos, q, len(q), arr, len(ops), jl, len(junction_lib),
      C.byref(params.c()), edit_dir, C.byref(s))
    return tuple(getattr(s, k) for k in STRICT_FIELDS)


def stitch_cigar(ops, p_start: int, bounds, junction_lens):
    """splice.rs:435-493; bounds [(pseudo_start, ref_start, ref_end)],
    junction_lens[i] = intron length of junction i; ops u32 (len << 4 | op)."""
    flat = [v for b in bounds for v in b]
    a = (C.c_uint32 * max(1, len(ops)))(*ops)
    bb = (C.c_uint32 * max(1, len(flat)))(*flat)
    jl = (C.c_uint32 * max(1, len(junction_lens)))(*junction_lens)
    cap = 2 * len(ops) + 2 * len(bounds) + 8
    out = (C.c_uint32 * cap)()
    f = lib().orc_stitch_cigar
    f.restype = C.c_uint32
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                  C.c_uint32, C.c_void_p, C.c_uint32]
    n = f(a, len(ops), p_start, bb, len(bounds), jl, len(junction_lens), out, cap)
    return list(out[:n])


def align_spliced_exons(contig: "Contig", read, exons, params: Params = Params()):
    """align_spliced (splice.rs:617-664) on the exon slices [(rs, re)]:
    (Ext against the pseudo-reference, stitched ops, genomic start)."""
    r = _b(read)
    total = sum(e - s for s, e in exons)
    flat = [v for x in exons for v in x]
    ex = (C.c_uint32 * max(1, len(flat)))(*flat)
    cap = 2 * (len(r) + total) + 8
    buf = (C.c_uint32 * cap)()
    e = _Ext(0, 0, 0, 0, 0, cap, buf)
    st = (C.c_uint32 * (cap + 2 * len(exons)))()
    ns, gs = C.c_uint32(), C.c_uint32()
    f = lib().orc_align_spliced_exons
    f.argtypes = [C.c_void_p, C.c_char_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    rc = f(C.byref(contig.c), r, len(r), ex, len(exons), C.byref(params.c()), C.byref(e), st,
           cap + 2 * len(exons), C.byref(ns), C.byref(gs))
    if rc != 0:
        raise OracleError(f"orc_align_spliced_exons returned {rc}")
    ext = Ext(e.read_start, e.read_end, e.ref_start, e.score, decode_ops(buf[:e.n_ops]))
    return ext, list(st[:ns.value]), gs.value


# ---- intron-chain fast path (intron_chain.rs:285-538) ----

class _LibEntry(C.Structure):
    _fields_ = [("contig", C.c_uint32), ("start", C.c_uint32), ("end", C.c_uint32),
                ("minus", C.c_int32), ("count", C.c_uint32)]


class _Frag(C.Structure):
    _fields_ = [("q_lo", C.c_uint32), ("q_hi", C.c_uint32), ("r_lo", C.c_uint32),
                ("r_hi", C.c_uint32), ("n_anchors", C.c_uint32)]


class _IntronParams(C.Structure):
    _fields_ = [("min_frag_cov", C.c_uint32), ("refine_window", C.c_uint32),
                ("refine_pattern_len", C.c_uint32), ("intron_max", C.c_uint32)]


class _IntronOut(C.Structure):
    _fields_ = [("found", C.c_int32), ("stage", C.c_int32), ("donor_end", C.c_uint32),
                ("acceptor_start", C.c_uint32), ("vd", C.c_int32), ("va", C.c_int32),
                ("junction", _Junction), ("signal", C.c_int32), ("support", C.c_uint32),
                ("left_start", C.c_uint32), ("right_end", C.c_uint32), ("ext", _Ext),
                ("stitched", C.POINTER(C.c_uint32)), ("stitched_cap", C.c_uint32),
                ("n_stitched", C.c_uint32)]


IC_STAGES = ("found", "empty", "anchors", "intron", "verify", "junction", "bounds", "result")


@dataclass
class IntronChain:
    found: bool
    stage: str
    donor_end: int
    acceptor_start: int
    vd: int
    va: int
    junction: Tuple[int, int, bool]
    signal: int
    support: int
    left_start: int
    right_end: int
    ext: Optional[Ext]
    cigar: List[Tuple[str, int]]


def intron_chain(contig: "Contig", contig_id: int, read, left, right, intron_start: int,
                 intron_end: int, minus: bool, junction_lib=(), params: Params = Params(),
                 refine_window: int = 30, refine_pattern_len: int = 50,
                 intron_max: int = 105_000) -> IntronChain:
    """try_intron_chain_placement (intron_chain.rs:392-538) from the best
    fragment pair on.  left / right: (q_lo, q_hi, r_lo, r_hi, n_anchors);
    junction_lib: (contig, start, end, minus, count) sorted as JunctionLib."""
    r = _b(read)
    jl = (_LibEntry * max(1, len(junction_lib)))(*[_LibEntry(*e) for e in junction_lib])
    ip = _IntronParams(15, refine_window, refine_pattern_len, intron_max)
    cap = 4 * len(r) + 64
    eops = (C.c_uint32 * cap)()
    sops = (C.c_uint32 * cap)()
    o = _IntronOut()
    o.ext.ops = eops
    o.ext.cap = cap
    o.stitched = sops
    o.stitched_cap = cap
    fn = lib().orc_intron_chain
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_char_p, C.c_uint32, C.POINTER(_Frag),
                  C.POINTER(_Frag), C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.c_uint64,
                  C.POINTER(_IntronParams), C.POINTER(_Params), C.POINTER(_IntronOut)]
    rc = fn(C.byref(contig.c), contig_id, r, len(r), C.byref(_Frag(*left)),
            C.byref(_Frag(*right)), intron_start, intron_end, int(minus), C.cast(jl, C.c_void_p),
            len(junction_lib), C.byref(ip), C.byref(params.c()), C.byref(o))
    if rc != 0:
        raise OracleError(f"orc_intron_chain returned {rc}")
    ext = None
    if o.stage in (0, 7):
        ext = Ext(o.ext.read_start, o.ext.read_end, o.ext.ref_start, o.ext.score,
                  decode_ops(eops[:o.ext.n_ops]))
    return IntronChain(bool(o.found), IC_STAGES[o.stage], o.donor_end, o.acceptor_start, o.vd,
                       o.va, (o.junction.start, o.junction.end, bool(o.junction.minus_strand)),
                       o.signal, o.support, o.left_start, o.right_end, ext,
                       decode_ops(sops[:o.n_stitched]) if o.stage in (0, 7) else [])
