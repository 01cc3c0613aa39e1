"""Host mirror of crates/map/src/extend.rs over the GB300 kernels.

Same names, argument meaning and results as the reference's public API:
``extend`` (extend.rs:347), ``extend_hint`` (:392), the parameter/result types
(:43-251), plus ``run_band`` (:606) for the kernel-equivalence checks the
reference's own tests perform.  Every call runs on the GPU through the C ABI
(include/esperanto_gb300.h); there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field
from enum import IntEnum
from typing import List, Optional, Tuple

from . import _native as N

# extend.rs:126
INITIAL_BAND = 30

OP_CHARS = "MIDNS"


class EditDir(IntEnum):
    """extend.rs:43-50: which A-to-I substitution scores 0."""
    Off = 0
    Ag = 1
    Tc = 2


@dataclass
class ExtendParams:
    """extend.rs:97-122 (mismatch stored negative, gap penalties positive)."""
    match_score: int = 2
    mismatch: int = -4
    gap_open: int = 4
    gap_ext: int = 2
    edit_dir: EditDir = EditDir.Off

    def _c(self) -> N.ExtendParamsC:
        return N.ExtendParamsC(self.match_score, self.mismatch, self.gap_open, self.gap_ext,
                               int(self.edit_dir))


@dataclass
class DiagHint:
    """extend.rs:190-198."""
    offset: int
    num: int = 1
    den: int = 1


@dataclass
class TouchRec:
    """extend.rs:216-229."""
    touched: bool = False
    row: int = 0
    left: bool = False
    clamped: bool = False


@dataclass
class Extension:
    """extend.rs:200-214; cigar is a list of (op char, length), S/M/I/D/N."""
    read_start: int
    read_end: int
    ref_start: int
    cigar: List[Tuple[str, int]] = field(default_factory=list)
    score: int = 0

    def key(self):
        return (self.score, self.read_start, self.read_end, self.ref_start, tuple(self.cigar))


def decode_cigar(ops) -> List[Tuple[str, int]]:
    return [(OP_CHARS[o & 15], o >> 4) for o in ops]


class ExtendBuffer:
    """Per-thread device context (extend.rs:231-251 ExtendBuffer): owns a CUDA
    stream, pinned staging and grow-only device scratch.  Not thread-safe; the
    reference likewise keeps one buffer per worker."""

    def __init__(self, device: int = 0):
        L = N.lib()
        h = C.c_void_p()
        rc = L.esp_create(C.byref(h), device)
        if rc != 0:
            raise N.EspError(rc, "esp_create failed (no CUDA device?)")
        self._h = h
        self._L = L

    @property
    def handle(self):
        return self._h

    def set_warp_max(self, warp_max: int):
        """Batches of at most warp_max pairs (and every per-call entry) run
        one warp per pair, larger ones one thread per pair; same results."""
        self.check(self._L.esp_set_warp_max(self._h, int(warp_max)))

    def set_kernel_variant(self, variant: int):
        """Thread-per-pair kernel variant: 0 / 1 one pair per thread (3 / 4
        blocks per SM), 2 / 3 two pairs of one band geometry per thread
        (band mode), -1 the default; same results."""
        self.check(self._L.esp_set_kernel_variant(self._h, int(variant)))

    def stream_ptr(self) -> int:
        return self._L.esp_stream(self._h) or 0

    def last_error(self) -> str:
        return self._L.esp_last_error(self._h).decode()

    def check(self, rc: int):
        if rc != 0:
            raise N.EspError(rc, self.last_error())

    def close(self):
        if getattr(self, "_h", None):
            self._L.esp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def _default_buffer() -> ExtendBuffer:
    buf = getattr(_tls, "buf", None)
    if buf is None:
        buf = _tls.buf = ExtendBuffer()
    return buf


def _b(x) -> bytes:
    return x.encode() if isinstance(x, str) else bytes(x)


def _call(fn, buf: Optional[ExtendBuffer], read, window, params: ExtendParams, *extra):
    buf = buf or _default_buffer()
    read, window = _b(read), _b(window)
    p = params._c()
    cap = 2 * (len(read) + len(window)) + 8
    ops = (C.c_uint32 * cap)()
    out = N.ExtensionC()
    rc = fn(buf.handle, read, len(read), window, len(window), C.byref(p), *extra, C.byref(out),
            ops, cap)
    buf.check(rc)
    ext = Extension(out.read_start, out.read_end, out.ref_start, decode_cigar(ops[:out.n_ops]),
                    out.score)
    touch = TouchRec(bool(out.touched), out.touch_row, bool(out.touch_left),
                     bool(out.touch_clamped))
    return ext, touch, bool(out.escalated)


def extend(read, ref_window, params: ExtendParams = ExtendParams(),
           buf: Optional[ExtendBuffer] = None) -> Extension:
    """extend.rs:347-354 full-window extension."""
    return _call(N.lib().esp_extend, buf, read, ref_window, params)[0]


def extend_hint(read, ref_window, params: ExtendParams = ExtendParams(),
                buf: Optional[ExtendBuffer] = None, hint: DiagHint = DiagHint(0),
                with_escalation: bool = False):
    """extend.rs:392-428 banded extension along a diagonal hint."""
    ext, _, esc = _call(N.lib().esp_extend_hint, buf, read, ref_window, params, hint.offset,
                        hint.num, hint.den)
    return (ext, esc) if with_escalation else ext


def run_band(read, ref_window, params: ExtendParams = ExtendParams(),
             buf: Optional[ExtendBuffer] = None,
             band: Optional[Tuple[int, int]] = None) -> Tuple[Extension, TouchRec]:
    """extend.rs:606-851 one kernel call; band = (offset, half) or None (full)."""
    off, half = band if band is not None else (0, -1)
    ext, touch, _ = _call(N.lib().esp_run_band, buf, read, ref_window, params, off, half)
    return ext, touch
