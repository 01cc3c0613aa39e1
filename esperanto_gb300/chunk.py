"""The pipeline batching hook (crates/map/src/pipeline.rs:394-403): a chunk
collector over the batch API.

The reference's chunk loop calls ``extend_hint`` / ``run_band`` / ``extend``
and the EA-Myers filters one read at a time from its rayon workers.  A
``Chunk`` gathers those calls instead -- from any number of threads, each
``add_*`` returning the request's index in input order -- and ``run`` sends
each kind through the batch API as one batch.  ``extension(i)`` /
``myers(i)`` then return exactly what the per-call entry point returns for
request i.  Reads whose later calls depend on earlier results run in rounds
(add, run, read, ``reset``).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

from . import _native as N
from .extend import (DiagHint, ExtendBuffer, ExtendParams, Extension, _b, _default_buffer,
                     decode_cigar)

MYERS_KINDS = {
    "myers_ea::infix": 0, "myers_ea::infix_best_end": 1, "myers_ea::infix_best_start": 2,
    "myers_ea::long::infix": 3, "myers_ea::long::infix_best_end": 4,
    "myers_ea::long::infix_best_start": 5, "engine::myers::infix": 6,
    "engine::myers::global": 7,
}


class Chunk:
    def __init__(self, buf: Optional[ExtendBuffer] = None, cigar_stride: int = 64):
        self.buf = buf or _default_buffer()
        self.stride = cigar_stride
        c = C.c_void_p()
        rc = N.lib().esp_chunk_create(self.buf.handle, cigar_stride, C.byref(c))
        if rc:
            raise N.EspError(rc, "esp_chunk_create")
        self._c = c

    def _add(self, fn, *args) -> int:
        idx = C.c_uint64()
        rc = fn(self._c, *args, C.byref(idx))
        if rc:
            raise N.EspError(rc, fn.__name__)
        return idx.value

    def add_extend_hint(self, read, window, hint: DiagHint) -> int:
        if hint.num != 1 or hint.den > 1:
            raise N.EspError(N.ESP_EINVAL, "DiagHint slope must be 1/1")
        read, window = _b(read), _b(window)
        return self._add(N.lib().esp_chunk_add_extend_hint, read, len(read), window,
                         len(window), hint.offset)

    def add_run_band(self, read, window, band: Optional[Tuple[int, int]] = None) -> int:
        read, window = _b(read), _b(window)
        off, half = band if band is not None else (0, -1)
        return self._add(N.lib().esp_chunk_add_run_band, read, len(read), window, len(window),
                         off, half)

    def add_extend(self, read, window) -> int:
        read, window = _b(read), _b(window)
        return self._add(N.lib().esp_chunk_add_extend, read, len(read), window, len(window))

    def add_myers(self, kind: str, read, text) -> int:
        read, text = _b(read), _b(text)
        return self._add(N.lib().esp_chunk_add_myers, MYERS_KINDS[kind], read, len(read), text,
                         len(text))

    def run(self, params: ExtendParams = ExtendParams()):
        p = params._c()
        self.buf.check(N.lib().esp_chunk_run(self._c, C.byref(p)))

    def extension(self, index: int) -> Extension:
        out = N.ExtensionC()
        ops = (C.c_uint32 * self.stride)()
        self.buf.check(N.lib().esp_chunk_extension(self._c, index, C.byref(out), ops,
                                                   self.stride))
        return Extension(out.read_start, out.read_end, out.ref_start,
                         decode_cigar(ops[:out.n_ops]), out.score)

    def myers(self, index: int) -> Tuple[int, int]:
        d, p = C.c_int32(), C.c_uint64()
        self.buf.check(N.lib().esp_chunk_myers(self._c, index, C.byref(d), C.byref(p)))
        return d.value, p.value

    def __len__(self) -> int:
        return int(N.lib().esp_chunk_size(self._c))

    def reset(self):
        self.buf.check(N.lib().esp_chunk_reset(self._c))

    def close(self):
        if getattr(self, "_c", None):
            N.lib().esp_chunk_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
