"""CPU-side checks of the C ABI library: it builds, loads and exports every
symbol include/esperanto_gb300.h declares (no device calls here)."""
import ctypes

from esperanto_gb300 import _native as N
from esperanto_gb300 import build


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = N.exported_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_dtypes_match_c_structs():
    from esperanto_gb300 import batch as B
    assert B.PAIR_DTYPE.itemsize == ctypes.sizeof(N.PairC)
    assert B.EXT_DTYPE.itemsize == ctypes.sizeof(N.ExtensionC)
