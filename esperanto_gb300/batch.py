"""Batch-submit API over the GB300 kernels (new beside the per-call drop-in).

A batch is a 2-bit packed arena (the reference's contig layout,
crates/map/src/fasta.rs:1-5) plus one ``esp_pair`` record per read x window
pair; non-ACGT bases are N intervals relative to their sequence.  The
numpy dtypes below are byte-for-byte the C structs of
include/esperanto_gb300.h.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .extend import ExtendBuffer, ExtendParams, _default_buffer

PAIR_DTYPE = np.dtype([("read_pos", "<u8"), ("win_pos", "<u8"), ("read_len", "<u4"),
                       ("win_len", "<u4"), ("band_offset", "<i4"), ("band_half", "<i4"),
                       ("n_first", "<u4"), ("n_read", "<u2"), ("n_win", "<u2")])
EXT_DTYPE = np.dtype([("read_start", "<u4"), ("read_end", "<u4"), ("ref_start", "<u4"),
                      ("score", "<i4"), ("n_ops", "<u4"), ("touch_row", "<i4"),
                      ("touched", "u1"), ("touch_left", "u1"), ("touch_clamped", "u1"),
                      ("escalated", "u1"), ("status", "<i4")])
NIV_DTYPE = np.dtype([("start", "<u4"), ("end", "<u4")])
MYERS_PAIR_DTYPE = np.dtype([("read_pos", "<u8"), ("text_pos", "<u8"), ("read_len", "<u4"),
                             ("text_len", "<u4"), ("n_first", "<u4"), ("n_read", "<u2"),
                             ("n_text", "<u2")])
MYERS_RES_DTYPE = np.dtype([("dist", "<i4"), ("status", "<i4"), ("pos", "<u8")])
assert PAIR_DTYPE.itemsize == 40 and EXT_DTYPE.itemsize == 32
assert MYERS_PAIR_DTYPE.itemsize == 32 and MYERS_RES_DTYPE.itemsize == 16
MYERS_BEST_END, MYERS_BEST_START, MYERS_GLOBAL = 0, 1, 2

MODE_BAND = N.MODE_BAND
MODE_HINT = N.MODE_HINT

_CODE = np.full(256, 4, np.uint8)
for _i, _c in enumerate(b"ACGT"):
    _CODE[_c] = _i
    _CODE[_c + 32] = _i
_ASCII = np.frombuffer(b"ACGTN", np.uint8)


def pack_codes(codes: np.ndarray) -> np.ndarray:
    """Pack 2-bit codes (values 0..3) MSB-first, 4 per byte, + 16 bytes pad."""
    n = len(codes)
    padded = np.zeros(((n + 3) // 4) * 4, np.uint8)
    padded[:n] = codes & 3
    q = padded.reshape(-1, 4)
    packed = (q[:, 0] << 6) | (q[:, 1] << 4) | (q[:, 2] << 2) | q[:, 3]
    return np.concatenate([packed.astype(np.uint8), np.zeros(16, np.uint8)])


def unpack_codes(arena: np.ndarray, pos: int, length: int) -> np.ndarray:
    idx = pos + np.arange(length, dtype=np.int64)
    return (arena[idx >> 2] >> (6 - 2 * (idx & 3))) & 3


def pack_ascii_pairs(reads: Sequence[bytes], windows: Sequence[bytes],
                     offsets: Sequence[int], halfs: Sequence[int]):
    """ASCII reads/windows -> (arena, pairs, n_iv) with N runs extracted."""
    seqs = []
    for r, w in zip(reads, windows):
        seqs.append(bytes(r))
        seqs.append(bytes(w))
    lens = np.array([len(s) for s in seqs], np.int64)
    starts = np.concatenate([[0], np.cumsum(lens)])[:-1]
    allb = np.frombuffer(b"".join(seqs), np.uint8) if seqs else np.zeros(0, np.uint8)
    codes = _CODE[allb]
    arena = pack_codes(codes)
    isn = codes == 4
    # N runs per sequence (runs never cross a sequence start)
    seq_start_mask = np.zeros(len(codes) + 1, bool)
    seq_start_mask[starts[lens > 0]] = True
    prev = np.concatenate([[False], isn[:-1]])
    run_start = np.nonzero(isn & (~prev | seq_start_mask[:-1]))[0]
    nxt = np.concatenate([isn[1:], [False]])
    run_end = np.nonzero(isn & (~nxt | seq_start_mask[1:]))[0] + 1
    sid = np.searchsorted(starts, run_start, side="right") - 1
    n_iv = np.zeros(len(run_start), NIV_DTYPE)
    n_iv["start"] = run_start - starts[sid]
    n_iv["end"] = run_end - starts[sid]
    counts = np.bincount(sid, minlength=len(seqs)) if len(seqs) else np.zeros(0, np.int64)
    first = np.concatenate([[0], np.cumsum(counts)])[:-1]
    npairs = len(reads)
    pairs = np.zeros(npairs, PAIR_DTYPE)
    pairs["read_pos"] = starts[0::2]
    pairs["win_pos"] = starts[1::2]
    pairs["read_len"] = lens[0::2]
    pairs["win_len"] = lens[1::2]
    pairs["band_offset"] = np.asarray(offsets, np.int64)
    pairs["band_half"] = np.asarray(halfs, np.int64)
    pairs["n_first"] = first[0::2]
    pairs["n_read"] = counts[0::2]
    pairs["n_win"] = counts[1::2]
    return arena, pairs, n_iv


def decode_pair(arena: np.ndarray, pair, n_iv: Optional[np.ndarray] = None) -> Tuple[bytes, bytes]:
    """ASCII read and window of one pair (N runs restored)."""
    r = _ASCII[unpack_codes(arena, int(pair["read_pos"]), int(pair["read_len"]))].copy()
    w = _ASCII[unpack_codes(arena, int(pair["win_pos"]), int(pair["win_len"]))].copy()
    if n_iv is not None and len(n_iv):
        f = int(pair["n_first"])
        for k in range(int(pair["n_read"])):
            r[n_iv[f + k]["start"]:n_iv[f + k]["end"]] = ord("N")
        f += int(pair["n_read"])
        for k in range(int(pair["n_win"])):
            w[n_iv[f + k]["start"]:n_iv[f + k]["end"]] = ord("N")
    return r.tobytes(), w.tobytes()


def cells_of(pairs: np.ndarray, mode: int = MODE_BAND, escalated: Optional[np.ndarray] = None) -> int:
    """DP cells (sum over rows of the in-window width, extend.rs:653-696)."""
    m = pairs["read_len"].astype(np.int64)
    n = pairs["win_len"].astype(np.int64)
    if mode == MODE_HINT:
        off = pairs["band_offset"].astype(np.int64)
        half = np.where(n <= 30, -1, 30)
        cells = _band_cells(m, n, off, half)
        if escalated is not None:
            cells = cells + np.where((n > 30) & (escalated != 0), m * n, 0)
        return int(cells.sum())
    return int(_band_cells(m, n, pairs["band_offset"].astype(np.int64),
                           pairs["band_half"].astype(np.int64)).sum())


def _band_cells(m, n, off, half):
    out = np.zeros(len(m), np.int64)
    full = half < 0
    out[full] = (m * n)[full]
    idx = np.nonzero(~full)[0]
    if len(idx) == 0:
        return out
    # group identical geometries (batches are highly repetitive)
    key = np.stack([m[idx], n[idx], off[idx], half[idx]], 1)
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    vals = np.zeros(len(uniq), np.int64)
    for u, (mm, nn, oo, hh) in enumerate(uniq):
        i = np.arange(1, mm + 1)
        c = np.clip(oo + i, 1, nn)
        lo = np.maximum(c - hh, 1)
        hi = np.minimum(c + hh, nn)
        vals[u] = int(np.maximum(hi - lo + 1, 0).sum())
    out[idx] = vals[inv.ravel()]
    return out


def extend_batch_host(pairs: np.ndarray, arena: np.ndarray, n_iv: Optional[np.ndarray] = None,
                      params: ExtendParams = ExtendParams(), mode: int = MODE_BAND,
                      cigar_stride: int = 64, buf: Optional[ExtendBuffer] = None):
    """End-to-end batch: host inputs -> device -> host results."""
    buf = buf or _default_buffer()
    pairs = np.ascontiguousarray(pairs, PAIR_DTYPE)
    arena = np.ascontiguousarray(arena, np.uint8)
    n_iv = np.zeros(0, NIV_DTYPE) if n_iv is None else np.ascontiguousarray(n_iv, NIV_DTYPE)
    out = np.zeros(len(pairs), EXT_DTYPE)
    cig = np.zeros(max(1, len(pairs) * cigar_stride), np.uint32)
    p = params._c()
    rc = N.lib().esp_batch_extend_host(buf.handle, mode, pairs.ctypes.data, len(pairs),
                                       arena.ctypes.data, len(arena),
                                       n_iv.ctypes.data if len(n_iv) else None, len(n_iv),
                                       C.byref(p), out.ctypes.data, cig.ctypes.data,
                                       cigar_stride)
    buf.check(rc)
    return out, cig[: len(pairs) * cigar_stride].reshape(len(pairs), cigar_stride)


def cigar_of(cig_row: np.ndarray, n_ops: int):
    return [("MIDNS"[int(o) & 15], int(o) >> 4) for o in cig_row[:n_ops]]


def pack_ascii_myers(reads, texts):
    """ASCII read/text pairs -> (arena, myers pairs, n_iv)."""
    arena, pp, n_iv = pack_ascii_pairs(reads, texts, [0] * len(reads), [0] * len(reads))
    pairs = np.zeros(len(pp), MYERS_PAIR_DTYPE)
    pairs["read_pos"] = pp["read_pos"]
    pairs["text_pos"] = pp["win_pos"]
    pairs["read_len"] = pp["read_len"]
    pairs["text_len"] = pp["win_len"]
    pairs["n_first"] = pp["n_first"]
    pairs["n_read"] = pp["n_read"]
    pairs["n_text"] = pp["n_win"]
    return arena, pairs, n_iv


def myers_batch_host(pairs, arena, n_iv=None, mode: int = MYERS_BEST_END,
                     buf: Optional[ExtendBuffer] = None):
    buf = buf or _default_buffer()
    pairs = np.ascontiguousarray(pairs, MYERS_PAIR_DTYPE)
    arena = np.ascontiguousarray(arena, np.uint8)
    n_iv = np.zeros(0, NIV_DTYPE) if n_iv is None else np.ascontiguousarray(n_iv, NIV_DTYPE)
    out = np.zeros(len(pairs), MYERS_RES_DTYPE)
    rc = N.lib().esp_batch_myers_host(buf.handle, mode, pairs.ctypes.data, len(pairs),
                                      arena.ctypes.data, len(arena),
                                      n_iv.ctypes.data if len(n_iv) else None, len(n_iv),
                                      out.ctypes.data)
    buf.check(rc)
    return out
