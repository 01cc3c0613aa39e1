"""Host mirror of crates/engine/src/myers.rs (the L1 verifier) over the GB300
Myers kernel: ``infix`` (myers.rs:32), ``global_`` (``global``, :42) and the
``long`` namespace (:45-63).  Pattern lengths 1..=256 (the reference asserts;
here EspError)."""
from __future__ import annotations

import ctypes as C
from types import SimpleNamespace
from typing import Optional

from . import _native as N
from .extend import ExtendBuffer, _b, _default_buffer


def _call(name, read, text, buf):
    buf = buf or _default_buffer()
    read, text = _b(read), _b(text)
    d = C.c_uint32()
    buf.check(getattr(N.lib(), name)(buf.handle, read, len(read), text, len(text), C.byref(d)))
    return d.value


def infix(read, text, buf: Optional[ExtendBuffer] = None) -> int:
    return _call("esp_engine_myers_infix", read, text, buf)


def global_(read, text, buf: Optional[ExtendBuffer] = None) -> int:
    return _call("esp_engine_myers_global", read, text, buf)


long = SimpleNamespace(infix=infix, global_=global_)
