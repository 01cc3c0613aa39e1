"""Serving loop (new): continuous batching of alignment requests over a
resident genome, behind the native server of csrc/serve.cpp.

``Server.submit`` hands a request (reads + their candidate windows) to the
native worker thread and returns at once; the worker turns the head of the
FIFO queue into launches of up to ``max_reads`` reads (small requests share
a launch, large ones run over several), each charged its DP scratch from one
pool of ``mem_budget`` bytes, so requests that arrive while others run
overlap on the device as slots and memory free up.  ``Server.wait`` returns the
request's status and its submit-to-results latency.  ``run_load`` drives a
server with Poisson arrivals for the serve benchmark.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _native as N
from . import batch as B
from .extend import ExtendParams
from .split import Genome

SERVE_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("contig", "<u4"),
                             ("win_start", "<u4"), ("win_len", "<u4"), ("hint_offset", "<i4"),
                             ("pad", "<u4")])


@dataclass
class Ticket:
    id: int
    reads: np.ndarray
    arena: np.ndarray
    out: np.ndarray
    cigar: np.ndarray
    stride: int


class Server:
    def __init__(self, genome: Genome, params: ExtendParams = ExtendParams(),
                 n_streams: int = 4, max_reads: int = 131072, max_read_len: int = 300,
                 mem_budget: int = 16 << 30, device: int = 0):
        self.genome = genome
        cfg = N.ServerConfigC(n_streams, max_reads, max_read_len, max_read_len + 128, mem_budget)
        p = params._c()
        s = C.c_void_p()
        rc = N.lib().esp_server_create(genome.handle, C.byref(p), C.byref(cfg), device,
                                       C.byref(s))
        if rc:
            raise N.EspError(rc, "esp_server_create")
        self._s = s

    def submit(self, arena: np.ndarray, reads: np.ndarray, cigar_stride: int = 32,
               out: Optional[np.ndarray] = None, cigar: Optional[np.ndarray] = None) -> Ticket:
        """Queue one request; results land in `out` / `cigar` (allocated here
        unless given: callers that recycle buffers pass their own)."""
        reads = np.ascontiguousarray(reads, SERVE_READ_DTYPE)
        arena = np.ascontiguousarray(arena, np.uint8)
        out = np.zeros(len(reads), B.EXT_DTYPE) if out is None else out
        cig = np.zeros(max(1, len(reads) * cigar_stride), np.uint32) if cigar is None else cigar
        if (out.dtype != B.EXT_DTYPE or len(out) < len(reads) or not out.flags.c_contiguous or
                cig.dtype != np.uint32 or len(cig) < len(reads) * cigar_stride or
                not cig.flags.c_contiguous):
            raise ValueError("result buffers too small or of the wrong type")
        req = N.ServeRequestC(arena.ctypes.data, len(arena), reads.ctypes.data, len(reads),
                              out.ctypes.data, cig.ctypes.data, cigar_stride)
        t = C.c_uint64()
        rc = N.lib().esp_server_submit(self._s, C.byref(req), C.byref(t))
        if rc:
            raise N.EspError(rc, "esp_server_submit")
        return Ticket(t.value, reads, arena, out, cig, cigar_stride)

    def wait(self, ticket: Ticket, timeout_ms: int = 60000):
        st, lat = C.c_int32(), C.c_double()
        rc = N.lib().esp_server_wait(self._s, ticket.id, timeout_ms, C.byref(st), C.byref(lat))
        if rc:
            raise N.EspError(rc, "esp_server_wait")
        return st.value, lat.value

    def stats(self) -> dict:
        """Admission and memory counters since creation (esp_server_stats)."""
        st = N.ServerStatsC()
        rc = N.lib().esp_server_get_stats(self._s, C.byref(st))
        if rc:
            raise N.EspError(rc, "esp_server_get_stats")
        return {k: getattr(st, k) for k, _ in N.ServerStatsC._fields_}

    def close(self):
        N.lib().esp_server_close(self._s)

    def destroy(self):
        if getattr(self, "_s", None):
            N.lib().esp_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def serve_pairs(reads: np.ndarray, contigs: np.ndarray) -> np.ndarray:
    """The esp_pair records the server builds for a request (for checks)."""
    pairs = np.zeros(len(reads), B.PAIR_DTYPE)
    c = contigs[reads["contig"]]
    ws = np.minimum(reads["win_start"], c["len"])
    we = np.minimum(ws.astype(np.int64) + reads["win_len"], c["len"])
    pairs["read_pos"] = reads["read_pos"]
    pairs["read_len"] = reads["read_len"]
    pairs["win_pos"] = c["base"] + ws
    pairs["win_len"] = we - ws
    pairs["band_offset"] = reads["hint_offset"]
    pairs["band_half"] = 30
    return pairs


def hint_cells(reads: np.ndarray, contigs: np.ndarray, out: np.ndarray) -> int:
    """DP cells of a served request (band attempt + full attempt if escalated)."""
    return B.cells_of(serve_pairs(reads, contigs), B.MODE_HINT, out["escalated"])


def run_load(server: Server, pool: List, rate_pairs_per_s: float, duration_s: float,
             seed: int = 0, closed_loop: bool = False):
    """Drive `server` with requests drawn from `pool` ((arena, reads) tuples).
    Open loop: Poisson arrivals at `rate_pairs_per_s` pairs/s for
    `duration_s`.  Closed loop (peak measurement): keep the server saturated.
    Returns (latencies_ms, pairs_done, wall_s, tickets)."""
    rng = np.random.default_rng(seed)
    mean_size = float(np.mean([len(r) for _, r in pool]))
    # one result buffer pair per pool entry, written once up front so that
    # results are copied into resident pages; two copies of one pool entry in
    # flight write identical bytes (the alignment of a request is fixed)
    bufs = []
    for _, r in pool:
        out, cig = np.empty(len(r), B.EXT_DTYPE), np.empty(max(1, len(r) * 32), np.uint32)
        out.view(np.uint8).fill(0)
        cig.fill(0)
        bufs.append((out, cig))
    lam = rate_pairs_per_s / mean_size  # requests per second
    tickets, lock = [], threading.Lock()
    done = threading.Event()
    lat, pairs_done, cells = [], [0], [0]

    def waiter():
        k = 0
        while True:
            with lock:
                have = k < len(tickets)
                t = tickets[k] if have else None
            if not have:
                if done.is_set():
                    with lock:
                        if k >= len(tickets):
                            return
                    continue
                time.sleep(0.0005)
                continue
            st, ms = server.wait(t, 120000)
            if st != 0:
                raise N.EspError(st, "served request failed")
            lat.append(ms)
            pairs_done[0] += len(t.reads)
            k += 1

    w = threading.Thread(target=waiter, daemon=True)
    w.start()
    t0 = time.perf_counter()
    next_t = t0
    k = 0
    while True:
        now = time.perf_counter()
        if now - t0 >= duration_s:
            break
        if closed_loop:
            with lock:
                inflight = len(tickets) - len(lat)
            if inflight >= 8:
                time.sleep(0.0002)
                continue
        else:
            if now < next_t:
                time.sleep(min(next_t - now, 0.002))
                continue
            next_t += rng.exponential(1.0 / lam)
        arena, reads = pool[k % len(pool)]
        out, cig = bufs[k % len(pool)]
        k += 1
        t = server.submit(arena, reads, 32, out, cig)
        with lock:
            tickets.append(t)
    done.set()
    w.join()
    wall = time.perf_counter() - t0
    return np.array(lat), pairs_done[0], wall, tickets
