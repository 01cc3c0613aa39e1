"""Strict rescoring of placements (crates/map/src/align.rs:1060-1165
``Aligner::rescore_with``) on the GPU, over a resident genome.

``rescore_batch`` scores many placements in one launch; ``rescore_with``
is the one-placement form with the reference's arguments (query, the
placement's contig / start / CIGAR, the exempted editing direction, the
junction library).  Results are ``StrictScore`` records (align.rs:188-211).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .extend import ExtendBuffer, ExtendParams, _b, _default_buffer
from .split import Genome

RESCORE_ITEM_DTYPE = np.dtype([("query_pos", "<u8"), ("query_len", "<u4"), ("contig", "<u4"),
                               ("pos", "<u4"), ("op_first", "<u4"), ("op_count", "<u4"),
                               ("edit_dir", "<i4")])
STRICT_DTYPE = np.dtype([("score", "<i4"), ("aligned", "<u4"), ("matches", "<u4"),
                         ("mm", "<u4"), ("ea_ag", "<u4"), ("ea_tc", "<u4"), ("ins", "<u4"),
                         ("del", "<u4"), ("clipped", "<u4"), ("n_splice", "<u4"),
                         ("splice_score", "<i4"), ("status", "<i4")])
LIB_DTYPE = np.dtype([("contig", "<u4"), ("start", "<u4"), ("end", "<u4"),
                      ("minus_strand", "<i4")])
_OPS = {"M": 0, "I": 1, "D": 2, "N": 3, "S": 4}


@dataclass
class StrictScore:
    """align.rs:188-211."""
    score: int = 0
    aligned: int = 0
    matches: int = 0
    mm: int = 0
    ea_ag: int = 0
    ea_tc: int = 0
    ins: int = 0
    dels: int = 0
    clipped: int = 0
    n_splice: int = 0
    splice_score: int = 0

    def key(self) -> Tuple[int, ...]:
        return (self.score, self.aligned, self.matches, self.mm, self.ea_ag, self.ea_tc,
                self.ins, self.dels, self.clipped, self.n_splice, self.splice_score)


def encode_cigar(cigar) -> List[int]:
    """[(op char, len)] -> u32 (len << 4 | op)."""
    return [(int(n) << 4) | _OPS[op] for op, n in cigar]


def intron_length_penalty(n: int) -> int:
    """splice.rs:119-121 through the kernel's threshold table."""
    return int(N.lib().esp_intron_length_penalty(n))


def rescore_batch(genome: Genome, items: np.ndarray, queries: np.ndarray, ops: np.ndarray,
                  junction_lib: Optional[np.ndarray] = None,
                  params: ExtendParams = ExtendParams(),
                  buf: Optional[ExtendBuffer] = None) -> np.ndarray:
    """StrictScore records (STRICT_DTYPE) of `items` (RESCORE_ITEM_DTYPE) over
    a query arena (ASCII bytes) and a CIGAR op array; junction_lib is
    LIB_DTYPE sorted by (contig, start, end)."""
    buf = buf or _default_buffer()
    items = np.ascontiguousarray(items, RESCORE_ITEM_DTYPE)
    queries = np.ascontiguousarray(queries, np.uint8)
    ops = np.ascontiguousarray(ops, np.uint32)
    lib = (np.zeros(0, LIB_DTYPE) if junction_lib is None
           else np.ascontiguousarray(junction_lib, LIB_DTYPE))
    out = np.zeros(len(items), STRICT_DTYPE)
    p = params._c()
    rc = N.lib().esp_batch_rescore_host(buf.handle, genome.handle, items.ctypes.data, len(items),
                                        queries.ctypes.data if len(queries) else None,
                                        len(queries), ops.ctypes.data if len(ops) else None,
                                        len(ops), lib.ctypes.data if len(lib) else None,
                                        len(lib), C.byref(p), None, out.ctypes.data)
    buf.check(rc)
    return out


def rescore_with(genome: Genome, query, contig: int, pos: int, cigar, edit_dir: int = 0,
                 junction_lib: Sequence[Tuple[int, int, int]] = (),
                 params: ExtendParams = ExtendParams(),
                 buf: Optional[ExtendBuffer] = None) -> StrictScore:
    """align.rs:1060-1165 for one placement; cigar as [(op char, len)]."""
    q = np.frombuffer(_b(query), np.uint8)
    ops = np.array(encode_cigar(cigar), np.uint32)
    it = np.zeros(1, RESCORE_ITEM_DTYPE)
    it[0] = (0, len(q), contig, pos, 0, len(ops), edit_dir)
    lib = np.zeros(len(junction_lib), LIB_DTYPE)
    for k, (c, s, e) in enumerate(sorted(junction_lib)):
        lib[k] = (c, s, e, 0)
    r = rescore_batch(genome, it, q, ops, lib, params, buf)[0]
    if r["status"] != 0:
        raise N.EspError(int(r["status"]), "rescore refused the placement")
    return StrictScore(*(int(r[k]) for k in ("score", "aligned", "matches", "mm", "ea_ag",
                                             "ea_tc", "ins", "del", "clipped", "n_splice",
                                             "splice_score")))
