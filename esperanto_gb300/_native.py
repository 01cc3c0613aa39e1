"""ctypes binding of the C ABI in include/esperanto_gb300.h.

The shared library is built in-tree (esperanto_gb300/_lib) by
esperanto_gb300.build.  There is no CPU fallback: if the library is missing
or fails to load, every entry point raises NativeUnavailable.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

ESP_OK = 0
ESP_EINVAL = -1
ESP_ECUDA = -2
ESP_ECAP = -3
ESP_EDOMAIN = -4
ESP_ENOMEM = -5
ESP_EBUSY = -6
ESP_ETIMEOUT = -7
ESP_ECLOSED = -8

MODE_BAND = 0
MODE_HINT = 1


class NativeUnavailable(RuntimeError):
    """The GB300 extension library is not built or cannot be loaded."""


class EspError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"esperanto_gb300 error {code}: {msg}")
        self.code = code


class ExtendParamsC(C.Structure):
    _fields_ = [("match_score", C.c_int32), ("mismatch", C.c_int32), ("gap_open", C.c_int32),
                ("gap_ext", C.c_int32), ("edit_dir", C.c_int32)]


class ExtensionC(C.Structure):
    _fields_ = [("read_start", C.c_uint32), ("read_end", C.c_uint32), ("ref_start", C.c_uint32),
                ("score", C.c_int32), ("n_ops", C.c_uint32), ("touch_row", C.c_int32),
                ("touched", C.c_uint8), ("touch_left", C.c_uint8),
                ("touch_clamped", C.c_uint8), ("escalated", C.c_uint8), ("status", C.c_int32)]


class PairC(C.Structure):
    _fields_ = [("read_pos", C.c_uint64), ("win_pos", C.c_uint64), ("read_len", C.c_uint32),
                ("win_len", C.c_uint32), ("band_offset", C.c_int32), ("band_half", C.c_int32),
                ("n_first", C.c_uint32), ("n_read", C.c_uint16), ("n_win", C.c_uint16)]


class MyersResultC(C.Structure):
    _fields_ = [("dist", C.c_int32), ("status", C.c_int32), ("pos", C.c_uint64)]


class ContigC(C.Structure):
    _fields_ = [("base", C.c_uint64), ("len", C.c_uint32), ("n_first", C.c_uint32),
                ("n_count", C.c_uint32), ("pad", C.c_uint32)]


class JunctionC(C.Structure):
    _fields_ = [("contig", C.c_uint32), ("start", C.c_uint32), ("end", C.c_uint32),
                ("minus_strand", C.c_int32)]


class SpliceParamsC(C.Structure):
    _fields_ = [("min_intron", C.c_uint32), ("max_intron", C.c_uint32),
                ("gt_ag_bonus", C.c_int32), ("gc_ag_bonus", C.c_int32),
                ("at_ac_bonus", C.c_int32), ("noncanonical_penalty", C.c_int32),
                ("known_bonus", C.c_int32), ("refine_radius", C.c_uint32)]


class PaidxInfoC(C.Structure):
    _fields_ = [("k", C.c_uint32), ("w", C.c_uint32), ("freq_cutoff", C.c_uint32),
                ("contig_count", C.c_uint32), ("kmer_count", C.c_uint64),
                ("positions_count", C.c_uint64), ("fasta_sha256", C.c_uint8 * 32),
                ("arena_bytes", C.c_uint64), ("n_iv_count", C.c_uint64),
                ("names_bytes", C.c_uint64)]


class RetryOutcomeC(C.Structure):
    _fields_ = [("found", C.c_int32), ("dro", C.c_uint32), ("left_win_lo", C.c_uint32),
                ("total", C.c_int32), ("left", ExtensionC), ("right", ExtensionC)]


class ServeRequestC(C.Structure):
    _fields_ = [("read_arena", C.c_void_p), ("read_arena_bytes", C.c_uint64),
                ("reads", C.c_void_p), ("n_reads", C.c_uint64), ("out", C.c_void_p),
                ("cigar", C.c_void_p), ("cigar_stride", C.c_uint32)]


class ServerConfigC(C.Structure):
    _fields_ = [("n_streams", C.c_uint32), ("max_reads", C.c_uint32),
                ("max_read_len", C.c_uint32), ("max_win_len", C.c_uint32),
                ("mem_budget_bytes", C.c_uint64)]


class ServerStatsC(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("launches", "reads", "merged_launches",
                                          "split_requests", "budget_waits", "cut_launches",
                                          "pool_bytes", "pool_peak_bytes")]


class BatchLimitsC(C.Structure):
    _fields_ = [("max_read_len", C.c_uint32), ("max_win_len", C.c_uint32),
                ("max_half", C.c_int32)]


_lib = None


def library_path() -> str:
    return _build.LIB


def lib():
    """Load (building first if stale) the extension library."""
    global _lib
    if _lib is not None:
        return _lib
    try:
        path = _build.build()
    except Exception as e:  # nvcc missing or failing: no silent fallback
        if os.path.exists(_build.LIB):
            path = _build.LIB
        else:
            raise NativeUnavailable(f"cannot build the GB300 extension: {e}") from e
    try:
        L = C.CDLL(path)
    except OSError as e:
        raise NativeUnavailable(f"cannot load {path}: {e}") from e
    vp, sz, u8p = C.c_void_p, C.c_size_t, C.c_char_p
    L.esp_create.argtypes = [C.POINTER(vp), C.c_int]
    L.esp_destroy.argtypes = [vp]
    L.esp_last_error.argtypes = [vp]
    L.esp_last_error.restype = C.c_char_p
    L.esp_stream.argtypes = [vp]
    L.esp_stream.restype = vp
    L.esp_last_launch_count.argtypes = [vp]
    L.esp_last_launch_count.restype = C.c_uint64
    ext_args = [vp, u8p, sz, u8p, sz, C.POINTER(ExtendParamsC)]
    L.esp_extend.argtypes = ext_args + [C.POINTER(ExtensionC), vp, C.c_uint32]
    L.esp_extend_hint.argtypes = ext_args + [C.c_int64, C.c_uint32, C.c_uint32,
                                             C.POINTER(ExtensionC), vp, C.c_uint32]
    L.esp_run_band.argtypes = ext_args + [C.c_int64, C.c_int64, C.POINTER(ExtensionC), vp,
                                          C.c_uint32]
    L.esp_score_tail_win.argtypes = ext_args + [C.POINTER(ExtensionC), vp, C.c_uint32]
    L.esp_batch_extend_host.argtypes = [vp, C.c_int, vp, C.c_uint64, vp, C.c_uint64, vp,
                                        C.c_uint64, C.POINTER(ExtendParamsC), vp, vp, C.c_uint32]
    L.esp_batch_extend_device.argtypes = [vp, C.c_int, vp, C.c_uint64, vp, C.c_uint64, vp,
                                          C.c_uint64, C.POINTER(BatchLimitsC),
                                          C.POINTER(ExtendParamsC), vp, vp, C.c_uint32, vp]
    for name in ("esp_myers_infix", "esp_myers_long_infix"):
        getattr(L, name).argtypes = [vp, u8p, sz, u8p, sz, C.POINTER(C.c_int32)]
    for name in ("esp_myers_infix_best_end", "esp_myers_infix_best_start",
                 "esp_myers_long_infix_best_end", "esp_myers_long_infix_best_start"):
        getattr(L, name).argtypes = [vp, u8p, sz, u8p, sz, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_uint64)]
    for name in ("esp_engine_myers_infix", "esp_engine_myers_global"):
        getattr(L, name).argtypes = [vp, u8p, sz, u8p, sz, C.POINTER(C.c_uint32)]
    L.esp_batch_myers_device.argtypes = [vp, C.c_int, vp, C.c_uint64, C.c_uint32, vp, C.c_uint64,
                                         vp, C.c_uint64, vp, vp]
    L.esp_batch_myers_host.argtypes = [vp, C.c_int, vp, C.c_uint64, vp, C.c_uint64, vp,
                                       C.c_uint64, vp]
    L.esp_genome_create.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint32, vp, C.c_uint64,
                                    C.POINTER(vp)]
    L.esp_genome_destroy.argtypes = [vp]
    L.esp_set_warp_max.argtypes = [vp, C.c_long]
    L.esp_set_kernel_variant.argtypes = [vp, C.c_int]
    L.esp_batch_spliced_host.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, vp,
                                         C.c_uint64, vp, C.c_uint64, C.POINTER(ExtendParamsC),
                                         vp, vp, vp, C.c_uint32]
    L.esp_intron_length_penalty.argtypes = [C.c_uint32]
    L.esp_intron_length_penalty.restype = C.c_int32
    L.esp_batch_rescore_host.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint64,
                                         vp, C.c_uint64, C.POINTER(ExtendParamsC), vp, vp]
    L.esp_batch_rescore_device.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, vp,
                                           C.c_uint64, vp, C.c_uint64,
                                           C.POINTER(ExtendParamsC), vp, vp, vp]
    L.esp_batch_autotune.argtypes = [vp, C.c_int, vp, C.c_uint64, vp, C.c_uint64, vp,
                                     C.c_uint64, C.POINTER(BatchLimitsC),
                                     C.POINTER(ExtendParamsC), vp, vp, C.c_uint32, vp, vp, vp]
    L.esp_paidx_scan.argtypes = [vp, C.c_uint64, C.POINTER(PaidxInfoC), C.c_char_p, sz]
    L.esp_paidx_contigs.argtypes = [vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint32, vp,
                                    C.c_uint64, vp, C.c_uint64]
    L.esp_genome_from_paidx.argtypes = [vp, vp, C.c_uint64, C.POINTER(vp)]
    L.esp_retry_tail_start.argtypes = [vp, vp, u8p, sz, C.c_uint32, C.POINTER(JunctionC), C.c_int,
                                       C.c_uint32, C.POINTER(SpliceParamsC),
                                       C.POINTER(ExtendParamsC), C.POINTER(RetryOutcomeC), vp, vp,
                                       C.c_uint32]
    L.esp_batch_splice_host.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint64,
                                        vp, C.c_uint64, C.POINTER(SpliceParamsC),
                                        C.POINTER(ExtendParamsC), vp, vp, C.c_uint32]
    L.esp_batch_splice_device.argtypes = [vp, vp, vp, C.c_uint64, C.c_uint32, vp, C.c_uint64,
                                          vp, C.c_uint64, vp, C.c_uint64,
                                          C.POINTER(SpliceParamsC), C.POINTER(ExtendParamsC),
                                          vp, vp, C.c_uint32, vp]
    L.esp_server_create.argtypes = [vp, C.POINTER(ExtendParamsC), C.POINTER(ServerConfigC),
                                    C.c_int, C.POINTER(vp)]
    L.esp_server_submit.argtypes = [vp, C.POINTER(ServeRequestC), C.POINTER(C.c_uint64)]
    L.esp_server_wait.argtypes = [vp, C.c_uint64, C.c_int, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_double)]
    L.esp_server_get_stats.argtypes = [vp, C.POINTER(ServerStatsC)]
    L.esp_chunk_create.argtypes = [vp, C.c_uint32, C.POINTER(vp)]
    L.esp_chunk_add_extend_hint.argtypes = [vp, u8p, sz, u8p, sz, C.c_int64,
                                            C.POINTER(C.c_uint64)]
    L.esp_chunk_add_run_band.argtypes = [vp, u8p, sz, u8p, sz, C.c_int64, C.c_int64,
                                         C.POINTER(C.c_uint64)]
    L.esp_chunk_add_extend.argtypes = [vp, u8p, sz, u8p, sz, C.POINTER(C.c_uint64)]
    L.esp_chunk_add_myers.argtypes = [vp, C.c_int, u8p, sz, u8p, sz, C.POINTER(C.c_uint64)]
    L.esp_chunk_run.argtypes = [vp, C.POINTER(ExtendParamsC)]
    L.esp_chunk_extension.argtypes = [vp, C.c_uint64, C.POINTER(ExtensionC), vp, C.c_uint32]
    L.esp_chunk_myers.argtypes = [vp, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]
    L.esp_chunk_size.argtypes = [vp]
    L.esp_chunk_size.restype = C.c_uint64
    L.esp_chunk_reset.argtypes = [vp]
    L.esp_chunk_destroy.argtypes = [vp]
    L.esp_server_close.argtypes = [vp]
    L.esp_server_destroy.argtypes = [vp]
    L.esp_last_cells.argtypes = [vp]
    L.esp_last_cells.restype = C.c_uint64
    _lib = L
    return L


def exported_symbols():
    """Names declared in include/esperanto_gb300.h (for the load test)."""
    import re
    hdr = os.path.join(_build.ROOT, "include", "esperanto_gb300.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:[\w ]+\*?\s*)\b(esp_\w+)\s*\(", text, re.M)))
