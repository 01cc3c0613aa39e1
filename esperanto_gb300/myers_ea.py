"""Host mirror of crates/map/src/myers_ea.rs over the GB300 Myers kernel.

Same names and results as the reference: ``infix`` (myers_ea.rs:118),
``infix_best_end`` (:138), ``infix_best_start`` / ``infix_best_start_into``
(:158-185) and the ``long`` namespace (:189-310).  Distances are editing-aware
(read G matches reference A, read C matches reference T).  Every call runs on
the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from types import SimpleNamespace
from typing import Optional, Tuple

from . import _native as N
from .extend import ExtendBuffer, _b, _default_buffer


def _call2(name, read, text, buf):
    buf = buf or _default_buffer()
    read, text = _b(read), _b(text)
    d, p = C.c_int32(), C.c_uint64()
    buf.check(getattr(N.lib(), name)(buf.handle, read, len(read), text, len(text), C.byref(d),
                                     C.byref(p)))
    return d.value, p.value


def _call1(name, read, text, buf):
    buf = buf or _default_buffer()
    read, text = _b(read), _b(text)
    d = C.c_int32()
    buf.check(getattr(N.lib(), name)(buf.handle, read, len(read), text, len(text), C.byref(d)))
    return d.value


def infix(read, text, buf: Optional[ExtendBuffer] = None) -> int:
    return _call1("esp_myers_infix", read, text, buf)


def infix_best_end(read, text, buf: Optional[ExtendBuffer] = None) -> Tuple[int, int]:
    return _call2("esp_myers_infix_best_end", read, text, buf)


def infix_best_start(read, text, buf: Optional[ExtendBuffer] = None) -> Tuple[int, int]:
    return _call2("esp_myers_infix_best_start", read, text, buf)


def infix_best_start_into(read, text, rread=None, rtext=None,
                          buf: Optional[ExtendBuffer] = None) -> Tuple[int, int]:
    """The reversed-copy buffers of the reference are unused scratch here."""
    return infix_best_start(read, text, buf)


long = SimpleNamespace(
    infix=lambda read, text, buf=None: _call1("esp_myers_long_infix", read, text, buf),
    infix_best_end=lambda read, text, buf=None: _call2("esp_myers_long_infix_best_end", read,
                                                       text, buf),
    infix_best_start=lambda read, text, buf=None: _call2("esp_myers_long_infix_best_start",
                                                         read, text, buf),
    infix_best_start_into=lambda read, text, rread=None, rtext=None, buf=None: _call2(
        "esp_myers_long_infix_best_start", read, text, buf),
)
