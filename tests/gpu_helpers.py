"""Shared GPU-vs-oracle comparison helpers."""
import functools

import oracle as O
from esperanto_gb300 import batch as B
from esperanto_gb300.extend import ExtendParams


@functools.lru_cache(maxsize=None)
def oracle_case(read, win, edit_dir, band, mode):
    """Oracle result of one case as (score, rs, re, fs, cigar, touch)."""
    p = O.Params(edit_dir=edit_dir)
    if mode == B.MODE_HINT:
        e = O.extend_hint(read, win, p, offset=band[0])
        return e.key(), None
    e, t = O.run_dispatch(read, win, p, band=band)
    return e.key(), t


_BUFS = {}


def kernel_buffer(kind):
    """A handle pinned to one DP kernel: 'warp' (warp per pair), 'thread'
    (thread per pair, length binned) or 'paired' (two pairs of one band
    geometry per thread, band mode); None = the size-based default."""
    if kind is None:
        return None
    if kind not in _BUFS:
        from esperanto_gb300.extend import ExtendBuffer
        b = ExtendBuffer()
        b.set_warp_max(1 << 40 if kind == "warp" else 0)
        if kind == "paired":
            b.set_kernel_variant(2)
        _BUFS[kind] = b
    return _BUFS[kind]


def gpu_batch(cases, edit_dir, mode=B.MODE_BAND, cigar_stride=None, kernel=None):
    """cases: list of (read, win, band or None).  One batch per call."""
    reads = [c[0] for c in cases]
    wins = [c[1] for c in cases]
    offs = [(c[2][0] if c[2] is not None else 0) for c in cases]
    halfs = [(c[2][1] if c[2] is not None else -1) for c in cases]
    arena, pairs, n_iv = B.pack_ascii_pairs(reads, wins, offs, halfs)
    if cigar_stride is None:
        cigar_stride = max(8, max(2 * (len(r) + len(w)) + 8 for r, w in zip(reads, wins)))
    out, cig = B.extend_batch_host(pairs, arena, n_iv, ExtendParams(edit_dir=edit_dir), mode,
                                   cigar_stride, buf=kernel_buffer(kernel))
    res = []
    for k in range(len(cases)):
        o = out[k]
        assert o["status"] == 0, (k, int(o["status"]))
        key = (int(o["score"]), int(o["read_start"]), int(o["read_end"]), int(o["ref_start"]),
               tuple(B.cigar_of(cig[k], int(o["n_ops"]))))
        touch = O.Touch(bool(o["touched"]), int(o["touch_row"]), bool(o["touch_left"]),
                        bool(o["touch_clamped"]))
        res.append((key, touch, bool(o["escalated"])))
    return res


def compare(cases, edit_dirs, mode=B.MODE_BAND, ctxs=None,
            kernels=("thread", "warp", "paired")):
    """Run cases grouped by edit_dir through GPU (each DP kernel) and the
    oracle; assert equality.  The paired kernel runs band-mode batches only
    (hint batches on that handle run the one-pair kernel)."""
    n = 0
    for kern in kernels:
        if kern == "paired" and mode != B.MODE_BAND:
            continue
        n = _compare(cases, edit_dirs, mode, ctxs, kern)
    return n


def _compare(cases, edit_dirs, mode, ctxs, kernel):
    by_dir = {}
    for k, (c, d) in enumerate(zip(cases, edit_dirs)):
        by_dir.setdefault(d, []).append(k)
    n = 0
    for d, idx in by_dir.items():
        got = gpu_batch([cases[k] for k in idx], d, mode, kernel=kernel)
        for k, g in zip(idx, got):
            read, win, band = cases[k]
            want, wt = oracle_case(read, win, d, band, mode)
            ctx = ctxs[k] if ctxs else str(k)
            assert g[0] == want, f"{ctx} [{kernel}]: gpu {g[0]} != oracle {want}"
            if wt is not None:
                assert g[1] == wt, f"{ctx} [{kernel}]: touch gpu {g[1]} != oracle {wt}"
            n += 1
    return n
