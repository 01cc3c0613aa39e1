"""Benchmark of the GB300 alignment inner loop (one JSON line on rank 0).

Default workload = the mixed-length batch:
4,194,304 read x window pairs, read length U[50,300], band half-width in
{16,32,64,128} w.p. {.4,.3,.2,.1}, windows of read + 2*half, banded affine DP
with full CIGAR traceback, in one persistent length-binned launch.  Other
workloads: --config 0 (plain 150 x 214 banded DP, 65,536 pairs), 1 (EA-Myers
150-bp query vs 200-bp text, 1,048,576 pairs), 3 (splice-rescue flank DP,
524,288 split reads over their candidate junctions), 4 (serve loop: see
esperanto_gb300/serve.py).  All inputs are seeded synthetic data (the
reference ships no dataset).

One step = one pass of the hot path over the whole batch.  Metric: GCUPS,
DP cells per second (cells = sum over rows of the in-window width of every
DP attempt run, crates/map/src/extend.rs:653-696; Myers counts m*n).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--config 0|1|2|3] [--pairs P]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import workloads as W  # noqa: E402  (seeded inputs; no library is loaded at import)

# Integer ops per cell of the DP recurrence in its scalar 32-bit form (E 3,
# F 3, tag clears 2, LUT select + diag add + floor 3, H key 3, H tag 1,
# traceback-bit selects 2, row max 1; the multiply-adds that accumulate the
# traceback words are not counted): the algorithmic work of one cell.  The
# two-pairs-per-thread kernel does it in 16-bit SIMD halves, two cells per
# 32-bit lane-op, so its roofline peak is twice the 32-bit lane-op rate.
OPS_PER_CELL = 18
# Myers: 10 32-bit logic/add/shift ops per 32-cell limb per text column.
MYERS_OPS_PER_CELL = 10.0 / 32.0
# ncu DRAM bytes (read + write) of the DP kernel per launch, from the
# committed summaries: the 150 x 214 banded batch (65,536 pairs, one launch)
# and the Myers batch (1,048,576 pairs, one launch); the mixed-length batch
# per DP cell, captured on a
# 524,288-pair case of the same distribution and scaled by cells.
TRAFFIC_BYTES = {0: 51.8e6 + 348.4e6, 1: 125.5e6 + 9.3e6}
# keyed by (workload, SIMD lanes): one pair per thread, two pairs per thread
TRAFFIC_PER_CELL = {(2, 1): (2713001472 + 6431804160) / 7716062109,
                    (2, 2): (35225117184 + 60432276480) / 61820954081}
TRAFFIC_SOURCE = {0: "profiles/gotoh_kernel_banded150x214_65536pairs.md",
                  1: "profiles/myers_kernel_150x200_1048576pairs.md",
                  2: "profiles/gotoh_kernel_traffic_mixedlength.md (scaled by cells)"}
DEFAULT_PAIRS = {0: 65536, 1: 1048576, 2: 4194304, 3: 524288}
SEEDS = {0: 1, 1: 2, 2: 3, 3: 4}


def int_peak(device, lanes=1):
    """Measured integer-ALU issue peak of this GPU (lane-ops/s): the slower
    of the 3-input-logic and integer-max probe streams (esp_probe_int_peaks);
    for the 16x2 SIMD kernel (lanes = 2) the slowest of those and the 16x2
    add-max / 3-way-max streams (esp_probe_simd16_peaks), times two 16-bit
    cells per lane-op."""
    import workloads as W
    lop3, imnmx, iadd, imad = W.int_peaks(device)
    probe = {"lop3": lop3 / 1e12, "imnmx": imnmx / 1e12, "iadd": iadd / 1e12,
             "imad": imad / 1e12}
    peak = min(lop3, imnmx)
    if lanes == 2:
        addmax, max3 = W.simd16_peaks(device)
        probe["addmax_s16x2"], probe["max3_s16x2"] = addmax / 1e12, max3 / 1e12
        peak = 2 * min(peak, addmax, max3)
    return peak, probe


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, device_index: int = 0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9 or f[0] != str(device_index):
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except Exception:
            pass
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workloads

class Workload:
    config = -1
    dtype = "int16"
    mode = ""
    ops_per_cell = OPS_PER_CELL

    def describe(self, n):
        raise NotImplementedError


class GotohWorkload(Workload):
    """The banded Gotoh batches (150 x 214 pairs; the mixed-length batch):
    run_band with traceback over a pair batch."""

    def __init__(self, config):
        self.config = config
        self.mode = "run_band"

    def describe(self, n):
        if self.config == 0:
            return (f"plain banded Gotoh: {n} pairs, 150-bp reads vs 214-bp windows, "
                    "band half 32 at offset 32, traceback to CIGAR")
        return (f"batched uneven Gotoh: {n} pairs, read U[50,300], half {{16,32,64,128}} "
                "w.p. {.4,.3,.2,.1}, window read+2*half, traceback to CIGAR")

    def setup(self, seed, n, dev, buf, torch):
        from esperanto_gb300 import _native as N
        from esperanto_gb300 import batch as B
        from esperanto_gb300.extend import ExtendParams
        L = N.lib()
        self.stride = 32
        arena, pairs = W.synth_gotoh(seed, n, self.config)
        self.cells = B.cells_of(pairs)
        self.n = n
        d_arena = torch.from_numpy(arena).to(dev)
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).to(dev)
        d_out = torch.empty(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        d_cig = torch.empty(n * self.stride, dtype=torch.int32, device=dev)
        lim = N.BatchLimitsC(int(pairs["read_len"].max()), int(pairs["win_len"].max()),
                             int(pairs["band_half"].max()))
        p = ExtendParams()._c()
        self._keep = (d_arena, d_pairs, d_out, d_cig, lim, p)
        self.autotune = None
        if n > 2048 and not getattr(self, "no_autotune", False):
            # pick the DP variant per length class on this batch (untimed);
            # timed steps then replay one captured graph of the tuned launches
            nv = 4  # kernel variants timed per class
            variants, ms = (C.c_int * 4)(), (C.c_double * (5 * nv))()
            buf.check(L.esp_batch_autotune(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n,
                                           d_arena.data_ptr(), arena.nbytes, None, 0,
                                           C.byref(lim), C.byref(p), d_out.data_ptr(),
                                           d_cig.data_ptr(), self.stride, None, variants, ms))
            self.autotune = {"classes": ["w>=196", "100<=w<196", "52<=w<100", "w<52",
                                         "whole list"],
                             "variants": list(variants),
                             "ms": [[round(ms[nv * s + v], 3) for v in range(nv)]
                                    for s in range(5)]}
            chosen = list(variants)
        else:  # the handle's default: by size unless ESP_GOTOH_VARIANT is set
            forced = os.environ.get("ESP_GOTOH_VARIANT")
            chosen = [int(forced) if forced else (3 if n >= (1 << 20) else 1)]
        # variants 2 / 3 compute two pairs per thread in 16-bit SIMD halves
        self.lanes = 2 if any(v >= 2 for v in chosen) else 1
        if self.lanes == 2:
            self.dtype = "int16x2"

        self._arena_bytes = arena.nbytes
        self._pairs = pairs

        def step():
            buf.check(L.esp_batch_extend_device(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n,
                                                d_arena.data_ptr(), arena.nbytes, None, 0,
                                                C.byref(lim), C.byref(p), d_out.data_ptr(),
                                                d_cig.data_ptr(), self.stride, None))
        self.step = step
        self.result_status = lambda: d_out.cpu().numpy().view(B.EXT_DTYPE)["status"]
        pin_arena = torch.from_numpy(arena).pin_memory().numpy()
        pin_pairs = torch.from_numpy(pairs.view(np.uint8)).pin_memory().numpy()
        out_pin = torch.empty(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8).pin_memory().numpy()
        cig_pin = torch.empty(n * self.stride, dtype=torch.int32).pin_memory().numpy()
        self._pins = (pin_arena, pin_pairs, out_pin, cig_pin)

        def e2e():
            buf.check(L.esp_batch_extend_host(buf.handle, B.MODE_BAND, pin_pairs.ctypes.data, n,
                                              pin_arena.ctypes.data, pin_arena.nbytes, None, 0,
                                              C.byref(p), out_pin.ctypes.data,
                                              cig_pin.ctypes.data, self.stride))
        self.e2e_step = e2e
        self.h2d = pin_arena.nbytes + pin_pairs.nbytes
        self.d2h = out_pin.nbytes + cig_pin.nbytes
        self.input_mb = arena.nbytes / 1e6

    def plain_per_call(self, seed, sample, buf):
        """The plain per-call drop-in (esp_run_band, host buffers, one pair per
        call, as the reference's callers invoke run_band/extend) on a sample
        of the same workload: pairs/s."""
        from esperanto_gb300 import _native as N
        from esperanto_gb300 import batch as B
        from esperanto_gb300.extend import ExtendParams
        L = N.lib()
        arena, pairs = W.synth_gotoh(seed, sample, self.config)
        cases = []
        for k in range(sample):
            r = B._ASCII[B.unpack_codes(arena, int(pairs["read_pos"][k]),
                                        int(pairs["read_len"][k]))].tobytes()
            w = B._ASCII[B.unpack_codes(arena, int(pairs["win_pos"][k]),
                                        int(pairs["win_len"][k]))].tobytes()
            cases.append((r, w, int(pairs["band_offset"][k]), int(pairs["band_half"][k])))
        p = ExtendParams()._c()
        out = N.ExtensionC()
        cap = 4096
        ops = (C.c_uint32 * cap)()
        fn = L.esp_run_band

        def one(c):
            buf.check(fn(buf.handle, c[0], len(c[0]), c[1], len(c[1]), C.byref(p), c[2], c[3],
                         C.byref(out), ops, cap))
        for c in cases[:16]:
            one(c)
        t = time.perf_counter()
        for c in cases:
            one(c)
        dt = time.perf_counter() - t
        return sample / dt, f"{sample} pairs of the same workload, one esp_run_band call each"

    def hint_measure(self, buf, torch, stream, steps=5):
        """extend_hint (extend.rs:392-428) over the same resident batch: the
        banded attempt, escalating to the full matrix on a touch or a low
        score.  Returns GCUPS (cells of both attempts), ms per call and the
        escalation rate."""
        from esperanto_gb300 import _native as N
        from esperanto_gb300 import batch as B
        L = N.lib()
        d_arena, d_pairs, d_out, d_cig, lim, p = self._keep
        hlim = N.BatchLimitsC(lim.max_read_len, lim.max_win_len, 30)

        def call():
            buf.check(L.esp_batch_extend_device(buf.handle, B.MODE_HINT, d_pairs.data_ptr(),
                                                self.n, d_arena.data_ptr(), self._arena_bytes,
                                                None, 0, C.byref(hlim), C.byref(p),
                                                d_out.data_ptr(), d_cig.data_ptr(), self.stride,
                                                None))
        for _ in range(3):
            call()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(stream)  # the handle's stream, where the kernels run
        for _ in range(steps):
            call()
        ev[1].record(stream)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / steps
        out = d_out.cpu().numpy().view(B.EXT_DTYPE)
        esc = out["escalated"]
        cells = B.cells_of(self._pairs, B.MODE_HINT, esc)
        return {"gcups": cells / (ms / 1e3) / 1e9, "ms_per_call": ms,
                "escalation_rate": float(esc.mean()), "cells_per_call": int(cells),
                "bad_status": int((out["status"] != 0).sum())}

    def cpu_reference(self, seed, sample, threads):
        import oracle as O
        from esperanto_gb300 import batch as B
        O.build()
        arena, pairs = W.synth_gotoh(seed, sample, self.config, lib=O.synth_lib())
        end = int((pairs["win_pos"] + pairs["win_len"]).max())
        seq = B._ASCII[B.unpack_codes(arena, 0, end)]

        def run():
            t = time.perf_counter()
            cells, _ = O.batch_extend(seq, pairs["read_pos"], pairs["read_len"], pairs["win_pos"],
                                      pairs["win_len"], pairs["band_offset"], pairs["band_half"],
                                      O.Params(), 0, threads)
            return cells, time.perf_counter() - t
        return run, f"{sample} pairs of the same workload per step"


class MyersWorkload(Workload):
    config = 1
    dtype = "u32"
    mode = "myers_ea::long::infix_best_end"
    ops_per_cell = MYERS_OPS_PER_CELL

    def describe(self, n):
        return (f"bit-parallel EA-Myers infix_best_end: {n} pairs, 150-bp query vs 200-bp "
                "text, 0-8 edits, 10% unrelated")

    def setup(self, seed, n, dev, buf, torch):
        from esperanto_gb300 import _native as N
        from esperanto_gb300 import batch as B
        L = N.lib()
        arena, pairs = W.synth_myers(seed, n)
        self.n = n
        self.cells = int((pairs["read_len"].astype(np.int64) * pairs["text_len"]).sum())
        d_arena = torch.from_numpy(arena).to(dev)
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).to(dev)
        d_out = torch.empty(n * B.MYERS_RES_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self._keep = (d_arena, d_pairs, d_out)

        def step():
            buf.check(L.esp_batch_myers_device(buf.handle, B.MYERS_BEST_END, d_pairs.data_ptr(),
                                               n, 150, d_arena.data_ptr(), arena.nbytes, None, 0,
                                               d_out.data_ptr(), None))
        self.step = step
        self.result_status = lambda: d_out.cpu().numpy().view(B.MYERS_RES_DTYPE)["status"]
        pin_arena = torch.from_numpy(arena).pin_memory().numpy()
        pin_pairs = torch.from_numpy(pairs.view(np.uint8)).pin_memory().numpy()
        out_pin = torch.empty(n * B.MYERS_RES_DTYPE.itemsize,
                              dtype=torch.uint8).pin_memory().numpy()
        self._pins = (pin_arena, pin_pairs, out_pin)

        def e2e():
            buf.check(L.esp_batch_myers_host(buf.handle, B.MYERS_BEST_END, pin_pairs.ctypes.data,
                                             n, pin_arena.ctypes.data, pin_arena.nbytes, None, 0,
                                             out_pin.ctypes.data))
        self.e2e_step = e2e
        self.h2d = pin_arena.nbytes + pin_pairs.nbytes
        self.d2h = out_pin.nbytes
        self.input_mb = arena.nbytes / 1e6

    def cpu_reference(self, seed, sample, threads):
        import oracle as O
        from esperanto_gb300 import batch as B
        O.build()
        sample *= 16
        arena, pairs = W.synth_myers(seed, sample, lib=O.synth_lib())
        end = int((pairs["text_pos"] + pairs["text_len"]).max())
        seq = B._ASCII[B.unpack_codes(arena, 0, end)]

        def run():
            t = time.perf_counter()
            cells, _, _ = O.batch_myers_best_end(seq, pairs["read_pos"], pairs["read_len"],
                                                 pairs["text_pos"], pairs["text_len"], threads)
            return cells, time.perf_counter() - t
        return run, f"{sample} pairs of the same workload per step"


class SpliceWorkload(Workload):
    config = 3
    mode = "split::channel_a (retry_tail_start per candidate)"

    def describe(self, n):
        return (f"splice-rescue flank DP: {n} 150-bp split reads (breakpoint U[20,130]), "
                "300-bp exon flanks, intron log-U[60,50k], true + decoy GT/AG candidates, "
                "11 breakpoints x 2 extend_hint per candidate")

    def setup(self, seed, n, dev, buf, torch):
        from esperanto_gb300 import _native as N
        from esperanto_gb300 import split as S
        from esperanto_gb300.extend import ExtendParams
        L = N.lib()
        garena, contigs, rarena, reads, cands = W.synth_splice(seed, n)
        self.n = n
        self.genome = S.Genome(garena, contigs, buf=buf)
        sp, p = S.SpliceParams()._c(), ExtendParams()._c()
        self.stride = 32
        # one host-API pass gives the DP cell census of the batch
        out, _, self.cells = S.channel_a_batch(self.genome, reads, rarena, cands,
                                               cigar_stride=self.stride, buf=buf)
        self.found = int(out["found"].sum())
        d_reads = torch.from_numpy(reads.view(np.uint8)).to(dev)
        d_arena = torch.from_numpy(rarena).to(dev)
        d_cands = torch.from_numpy(cands.view(np.uint8)).to(dev)
        d_out = torch.empty(n * S.SPLICE_RES_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        d_cig = torch.empty(n * self.stride, dtype=torch.int32, device=dev)
        self._keep = (d_reads, d_arena, d_cands, d_out, d_cig, sp, p)

        def step():
            buf.check(L.esp_batch_splice_device(buf.handle, self.genome.handle,
                                                d_reads.data_ptr(), n, 150, d_arena.data_ptr(),
                                                rarena.nbytes, None, 0, d_cands.data_ptr(),
                                                len(cands), C.byref(sp), C.byref(p),
                                                d_out.data_ptr(), d_cig.data_ptr(), self.stride,
                                                None))
        self.step = step
        self.result_status = lambda: d_out.cpu().numpy().view(S.SPLICE_RES_DTYPE)["status"]
        pin = [torch.from_numpy(a.view(np.uint8) if a.dtype != np.uint8 else a).pin_memory()
               .numpy() for a in (reads, rarena, cands)]
        out_pin = torch.empty(n * S.SPLICE_RES_DTYPE.itemsize, dtype=torch.uint8).pin_memory().numpy()
        cig_pin = torch.empty(n * self.stride, dtype=torch.int32).pin_memory().numpy()
        self._pins = (pin, out_pin, cig_pin)

        def e2e():
            buf.check(L.esp_batch_splice_host(buf.handle, self.genome.handle, pin[0].ctypes.data,
                                              n, pin[1].ctypes.data, pin[1].nbytes, None, 0,
                                              pin[2].ctypes.data, len(cands), C.byref(sp),
                                              C.byref(p), out_pin.ctypes.data,
                                              cig_pin.ctypes.data, self.stride))
        self.e2e_step = e2e
        self.h2d = sum(a.nbytes for a in pin)
        self.d2h = out_pin.nbytes + cig_pin.nbytes
        self.input_mb = (garena.nbytes + rarena.nbytes) / 1e6
        self.n_cands = len(cands)
        # the flank DPs (22 extend_hint pairs per candidate) run as one hint
        # batch: on the 16x2 paired kernel from 2^20 pairs unless overridden
        forced = os.environ.get("ESP_GOTOH_HINT_VARIANT")
        paired = int(forced) >= 2 if forced else 22 * len(cands) >= (1 << 20)
        self.lanes = 2 if paired else 1
        if paired:
            self.dtype = "int16x2"

    def cpu_reference(self, seed, sample, threads):
        import oracle as O
        from esperanto_gb300 import batch as B
        from esperanto_gb300 import split as S
        O.build()
        sample = max(64, sample // 16)
        garena, contigs, rarena, reads, cands = W.synth_splice(seed, sample, lib=O.synth_lib())
        ra = B._ASCII[B.unpack_codes(rarena, 0, len(reads) * 150)]

        def run():
            t = time.perf_counter()
            _, _, cells = O.batch_channel_a(garena, contigs, ra, reads["read_pos"], reads, cands,
                                            threads)
            return cells, time.perf_counter() - t
        return run, f"{sample} split reads of the same workload per step"


def serve_phase(args, device=0, clocked=True):
    """The serving workload: the serving loop on a resident synthetic genome
    (3.1 Gbp by default).  Measures the saturated throughput (closed loop),
    then Poisson arrivals of 1k-64k-read requests (log-uniform) at 70% and
    80% of it, reporting p50/p99 latency, with nvidia-smi clock samples over
    the loaded phases, the integer roofline at peak and the oracle's
    extend_hint on the same kind of reads as the CPU baseline."""
    from esperanto_gb300 import serve as SV
    from esperanto_gb300.extend import ExtendBuffer
    from esperanto_gb300.split import Genome
    buf = ExtendBuffer(device)
    t0 = time.perf_counter()
    garena, contigs = W.synth_genome(5, args.genome_bases, 24)
    genome = Genome(garena, contigs, buf=buf)
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(65536), args.pool)).astype(int)
    pool = [W.synth_request(5, k, garena, contigs, int(n)) for k, n in enumerate(sizes)]
    srv = SV.Server(genome, n_streams=args.streams, max_reads=65536, mem_budget=16 << 30,
                    device=device)
    # warm up every slot
    for t in [srv.submit(*pool[k % len(pool)]) for k in range(2 * args.streams)]:
        srv.wait(t)
    clk = ClockSampler()
    if clocked:
        clk.start()
    peak_s = max(1.0, args.serve_seconds / 2)
    lat, pairs, wall, tks = SV.run_load(srv, pool, 0, peak_s, closed_loop=True)
    peak = pairs / wall
    cells = sum(SV.hint_cells(t.reads, contigs, t.out) for t in tks)
    peak_gcups = cells / wall / 1e9
    res = {}
    for frac in (0.7, 0.8):
        lat, pairs, wall, tks = SV.run_load(srv, pool, frac * peak, args.serve_seconds, seed=7)
        res[f"{int(frac * 100)}pct"] = {
            "offered_pairs_per_s": frac * peak, "achieved_pairs_per_s": pairs / wall,
            "requests": len(lat), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max())}
    clocks = clk.stop(device) if clocked else None
    srv.destroy()
    out = {"workload": "serve loop: %.2f-Gbp resident genome (24 contigs), Poisson requests of "
                       "1k-64k reads (log-uniform), 2x150 PE, windows read +- 32, extend_hint "
                       "policy" % (args.genome_bases / 1e9),
           "streams": args.streams, "request_pool": args.pool,
           "peak_pairs_per_s": peak, "peak_gcups": peak_gcups, "peak_seconds": peak_s,
           "load": res, "load_seconds": args.serve_seconds, "setup_s": setup_s,
           "clocks": clocks}
    if clocked:
        peak_ops, _ = int_peak(device, 1)
        out["roofline"] = {"bound": "int_alu",
                           "achieved": peak_gcups * 1e9 * OPS_PER_CELL / 1e12,
                           "peak": peak_ops / 1e12, "unit": "Tops/s",
                           "frac": peak_gcups * 1e9 * OPS_PER_CELL / peak_ops,
                           "note": "saturated serve throughput (one pair per thread kernel)"}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = serve_cpu_baseline(garena, contigs, pool[0])
    return out


def serve_cpu_baseline(garena, contigs, request):
    """The oracle's extend_hint (the reference's scalar path) over one
    served request's reads on all host cores: GCUPS and pairs/s."""
    import oracle as O
    from esperanto_gb300 import batch as B
    from esperanto_gb300 import serve as SV
    arena, reads = request
    pairs = SV.serve_pairs(reads, contigs)
    idx = np.arange(len(reads))
    win_lo = int(pairs["win_pos"].min())
    win_hi = int((pairs["win_pos"] + pairs["win_len"]).max())
    # the reads, then the genome span their windows fall in, as one ASCII run
    rseq = B._ASCII[B.unpack_codes(arena, 0, len(reads) * 150)]
    gseq = B._ASCII[B.unpack_codes(garena, win_lo, win_hi - win_lo)]
    seq = np.concatenate([rseq, gseq])
    threads = os.cpu_count() or 1

    def run():
        t = time.perf_counter()
        cells, _ = O.batch_extend(seq, pairs["read_pos"][idx], pairs["read_len"][idx],
                                  pairs["win_pos"][idx] - win_lo + len(rseq),
                                  pairs["win_len"][idx], pairs["band_offset"][idx],
                                  pairs["band_half"][idx], O.Params(), 1, threads)
        return cells, time.perf_counter() - t
    run()
    cells, dt = run()
    return {"value": cells / dt / 1e9, "unit": "GCUPS", "pairs_per_s": len(idx) / dt,
            "cores": threads, "kind": "port",
            "sample": f"one served request of {len(idx)} reads through the oracle's "
                      "extend_hint (the reference's scalar code path on aarch64)"}


def serve_bench(args):
    """--config 4: the serve phase alone, as its own JSON line."""
    import torch
    torch.cuda.set_device(0)
    sv = serve_phase(args, 0)
    r70 = sv["load"]["70pct"]
    line = {"metric": "serve p99 latency at 70% of peak load", "value": r70["p99_ms"],
            "unit": "ms", "n_gpus": 1, "higher_is_better": False, "data": "synthetic",
            "dtype": "int16", "vs_baseline": None,
            "config": {"workload": sv["workload"], "streams": args.streams,
                       "request_pool": args.pool},
            "peak_pairs_per_s": sv["peak_pairs_per_s"], "peak_gcups": sv["peak_gcups"],
            "load": sv["load"], "setup_s": sv["setup_s"], "clocks": sv["clocks"],
            "roofline": sv.get("roofline"), "cpu_baseline": sv.get("cpu_baseline")}
    print(json.dumps(line), flush=True)


def other_config(config, args, local, torch):
    """A short, clocked measurement of another workload for the default line:
    the 150 x 214 banded batch (0), the EA-Myers batch (1) or the split-read
    rescue (3), each at its full size with inputs resident, end to end
    through the host batch API, on its own integer roofline and next to the
    oracle port on the host cores."""
    from esperanto_gb300 import _native as N
    from esperanto_gb300.extend import ExtendBuffer
    L = N.lib()
    dev = f"cuda:{local}"
    wl = make_workload(config)
    n = DEFAULT_PAIRS[config]
    seed = SEEDS[config]
    buf = ExtendBuffer(local)
    stream = torch.cuda.ExternalStream(buf.stream_ptr())
    wl.setup(seed, n, dev, buf, torch)
    for _ in range(3):
        wl.step()
    torch.cuda.synchronize()
    bad = int((wl.result_status() != 0).sum())
    steps = 3 if config == 3 else 10
    clk = ClockSampler()
    clk.start()
    t_clk = time.perf_counter()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with torch.cuda.stream(stream):
        evs[0].record(stream)
        for _ in range(steps):
            wl.step()
        evs[1].record(stream)
    torch.cuda.synchronize()
    while time.perf_counter() - t_clk < 0.6:  # let the 200 ms samples see the load
        wl.step()
        torch.cuda.synchronize()
    clocks = clk.stop(local)
    ms = evs[0].elapsed_time(evs[1]) / steps
    launches = int(L.esp_last_launch_count(buf.handle)) * steps
    e2e_ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        wl.e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    lanes = getattr(wl, "lanes", 1)
    peak_ops, _ = int_peak(local, lanes)
    achieved = wl.cells * wl.ops_per_cell / (ms / 1e3)
    out = {"workload": wl.describe(n), "metric": "GCUPS",
           "value": wl.cells / (ms / 1e3) / 1e9, "unit": "GCUPS", "ms_per_step": ms,
           "steps": steps, "warmup": 3, "pairs_per_s": n / (ms / 1e3), "dtype": wl.dtype,
           "cells_per_step": wl.cells, "bad_status": bad, "gpu_launches": launches,
           "e2e": {"value": wl.cells / (float(np.median(e2e_ms)) / 1e3) / 1e9, "unit": "GCUPS",
                   "h2d_bytes_per_step": int(wl.h2d), "d2h_bytes_per_step": int(wl.d2h),
                   "statistic": "median of 3 steps"},
           "roofline": {"bound": "int_alu", "achieved": achieved / 1e12,
                        "peak": peak_ops / 1e12, "unit": "Tops/s", "frac": achieved / peak_ops,
                        "ops_per_cell": wl.ops_per_cell, "simd_lanes": lanes},
           "clocks": clocks}
    if config == 0:
        out["extend_hint"] = wl.hint_measure(buf, torch, stream)
    if config == 3:
        out["candidates"] = wl.n_cands
        out["rescued"] = wl.found
    if not args.no_cpu_baseline:
        run, sample = wl.cpu_reference(seed, args.cpu_sample, os.cpu_count() or 1)
        run()
        c, dt = run()
        out["cpu_baseline"] = {"value": c / dt / 1e9, "unit": "GCUPS",
                               "cores": os.cpu_count() or 1, "kind": "port", "sample": sample}
    del wl
    buf.close()
    torch.cuda.empty_cache()
    return out


def make_workload(config):
    if config == 1:
        return MyersWorkload()
    if config == 3:
        return SpliceWorkload()
    return GotohWorkload(config)


# ---------------------------------------------------------------- main

def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if args.impl == "gpu" else "gloo")
    return rank, world, local


def reduce_over_ranks(ms, cells, e2e_s, e2e_cells, world, device="cpu"):
    """Whole-job figures of a weak-scaling run: the slowest rank's time and
    the units all ranks processed (kernel-timed and end-to-end legs)."""
    import torch
    t = torch.tensor([ms, e2e_s], dtype=torch.float64, device=device)
    c = torch.tensor([float(cells), float(e2e_cells)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t[0]), float(c[0]), float(t[1]), float(c[1])


def repo_libraries():
    """Shared libraries of this repository mapped into the process (paths
    relative to the repository), or None where /proc is unavailable."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return None
    root = os.path.realpath(ROOT)
    return sorted(os.path.relpath(p, root) for p in paths
                  if os.path.realpath(p).startswith(root + os.sep))


def reference_arm(args, wl, seed, threads, n_pairs):
    run, sample = wl.cpu_reference(seed, args.cpu_sample, threads)
    for _ in range(args.warmup):
        run()
    tot_cells, tot_t = 0, 0.0
    for _ in range(args.steps):
        c, dt = run()
        tot_cells += c
        tot_t += dt
    v = tot_cells / tot_t / 1e9
    line = {"metric": "GCUPS", "value": v, "unit": "GCUPS", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic",
            "config": {"workload": wl.describe(n_pairs), "sample": sample},
            "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            # evidence that the arm ran the oracle port alone: no library of
            # the GPU path (or of the benchmark tooling) is mapped
            "repo_libraries_loaded": repo_libraries()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1,
                    help="GPUs of the node (one rank each under torchrun; replicas)")
    ap.add_argument("--steps", type=int, default=5, help="timed steps")
    ap.add_argument("--warmup", type=int, default=3, help="untimed warm-up steps")
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"],
                    help="reference: the oracle port of the reference on the host cores")
    ap.add_argument("--config", type=int, default=2, choices=[0, 1, 2, 3, 4],
                    help="0 banded 150x214, 1 Myers, 2 mixed-length (headline), "
                         "3 split-read rescue, 4 serve loop")
    ap.add_argument("--genome-bases", type=int, default=3_100_000_000,
                    help="resident genome of the serve workload")
    ap.add_argument("--pool", type=int, default=48, help="serve: distinct requests generated")
    ap.add_argument("--streams", type=int, default=4, help="serve: launch slots")
    ap.add_argument("--serve-seconds", type=float, default=4.0,
                    help="seconds at each of 70%% and 80%% of peak in the serve phase")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the serve phase of the default (mixed-length) line")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the other workloads' measurements in the default line")
    ap.add_argument("--pairs", type=int, default=0,
                    help="pairs (reads) of the workload; 0 = its full size")
    ap.add_argument("--cpu-sample", type=int, default=16384,
                    help="pairs per step of the CPU baseline / reference arm")
    ap.add_argument("--e2e-steps", type=int, default=8,
                    help="end-to-end steps through the host API (median reported)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the oracle-port CPU baseline of the line")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the per-length-class kernel autotuning (profiling runs)")
    args = ap.parse_args()
    rank, world, local = dist_init(args)
    config = args.config
    if config == 4:
        if rank == 0 and args.impl == "gpu":
            serve_bench(args)
        return
    n_pairs = args.pairs or DEFAULT_PAIRS[config]
    seed = SEEDS[config] + 1000 * rank  # weak scaling: each rank runs its own batch
    threads = os.cpu_count() or 1
    wl = make_workload(config)
    wl.no_autotune = args.no_autotune

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, wl, seed, threads, n_pairs)
        return

    import torch
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    from esperanto_gb300 import _native as N
    from esperanto_gb300.extend import ExtendBuffer
    L = N.lib()
    buf = ExtendBuffer(local)
    stream = torch.cuda.ExternalStream(buf.stream_ptr())
    wl.setup(seed, n_pairs, dev, buf, torch)

    warmup = max(3, args.warmup)
    for _ in range(warmup):
        wl.step()
    torch.cuda.synchronize()
    bad = int((wl.result_status() != 0).sum())
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    t_clk = time.perf_counter()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with torch.cuda.stream(stream):
        evs[0].record(stream)
        for k in range(args.steps):
            wl.step()
            evs[k + 1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    # nvidia-smi samples every 200 ms: a shorter timed region is followed by
    # untimed steps of the same work so that the samples see that load
    extended = False
    while time.perf_counter() - t_clk < 0.6:
        wl.step()
        torch.cuda.synchronize()
        extended = True
    clocks = clk.stop(local)
    if clocks is not None and extended:
        clocks["window"] = ("the timed region plus untimed steps of the same work "
                            "(0.6 s of sampling)")
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = sum(per_step) / args.steps
    launches = int(L.esp_last_launch_count(buf.handle)) * args.steps

    wl.e2e_step()
    e2e_ms = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        wl.e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = float(np.median(e2e_ms)) / 1e3  # host-side noise: median of the steps
    ms_max, cells_all, e2e_max, e2e_cells_all = reduce_over_ranks(ms, wl.cells, e2e_s, wl.cells,
                                                                  world, dev)
    value = cells_all / (ms_max / 1e3) / 1e9
    e2e_val = e2e_cells_all / e2e_max / 1e9
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if rank != 0:
        return

    peaks, src = load_peaks()
    lanes = getattr(wl, "lanes", 1)
    peak_ops, probe = int_peak(local, lanes)
    achieved_ops = wl.cells * wl.ops_per_cell / (ms / 1e3)
    traffic = None
    if config in TRAFFIC_BYTES and n_pairs == DEFAULT_PAIRS[config]:
        traffic = TRAFFIC_BYTES[config]
    elif (config, lanes) in TRAFFIC_PER_CELL:
        traffic = TRAFFIC_PER_CELL[(config, lanes)] * wl.cells
    plain = None
    if hasattr(wl, "plain_per_call"):
        pps, sample = wl.plain_per_call(seed, 2000, buf)
        batched_pps = n_pairs / (ms / 1e3)
        plain = {"pairs_per_s": pps, "sample": sample,
                 "batched_pairs_per_s": batched_pps, "batched_over_plain": batched_pps / pps}
    cpu = None
    if not args.no_cpu_baseline:
        run, sample = wl.cpu_reference(seed, args.cpu_sample, threads)
        run()
        c, dt = run()
        cpu = {"value": c / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
               "sample": sample + " (oracle restatement of the reference's scalar kernel, "
                                  "the code path the reference runs on aarch64)"}
    line = {
        "metric": "GCUPS", "value": value, "unit": "GCUPS", "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
        "data": "synthetic",
        "config": {"workload": wl.describe(n_pairs), "pairs": n_pairs,
                   "cells_per_step": wl.cells, "mode": wl.mode,
                   "l2": "inputs larger than L2 (%.0f MB of sequence + DP scratch)"
                         % wl.input_mb},
        "pairs_per_s": n_pairs * world / (ms_max / 1e3),
        "bad_status": bad,
        "gpu_launches": launches,
        "roofline": {"bound": "int_alu", "achieved": achieved_ops / 1e12,
                     "hbm_achieved_gbs": (traffic / (ms / 1e3) / 1e9) if traffic else None,
                     "hbm_frac": (traffic / (ms / 1e3) / 1e9 / peaks["hbm_gbs"])
                     if traffic and peaks.get("hbm_gbs") else None,
                     "peak": peak_ops / 1e12, "unit": "Tops/s",
                     "frac": achieved_ops / peak_ops, "traffic": traffic,
                     "traffic_source": TRAFFIC_SOURCE.get(config),
                     "peak_source": "measured on this GPU (esp_probe_int_peaks: independent streams "
                                    "of 3-input logic / integer max, the ALU-pipe issue rate)"
                                    + ("; with the 16x2 add-max / 3-way-max streams "
                                       "(esp_probe_simd16_peaks) for the two-pairs-per-thread "
                                       "kernel, x 2 cells per lane-op" if lanes == 2 else ""),
                     "simd_lanes": lanes,
                     "probe_tops": probe, "ops_per_cell": wl.ops_per_cell,
                     "hbm_peak_gbs": peaks.get("hbm_gbs"), "hbm_peak_source": src},
        "plain_per_call": plain,
        "e2e": {"value": e2e_val, "unit": "GCUPS", "h2d_bytes_per_step": int(wl.h2d),
                "d2h_bytes_per_step": int(wl.d2h), "ms_per_step": [round(x, 3) for x in e2e_ms],
                "statistic": f"median of {len(e2e_ms)} steps"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "per_step_ms": per_step,
    }
    if getattr(wl, "autotune", None):
        line["config"]["autotune"] = wl.autotune
        line["config"]["cuda_graph"] = "timed steps replay one captured graph"
    if config == 3:
        line["config"]["candidates"] = wl.n_cands
        line["config"]["rescued"] = wl.found
    if config in (0, 2):
        # the same pairs through extend_hint, the policy the reference's
        # callers run (align.rs:1907): its escalation rate is how often the
        # two-attempt policy runs twice
        line["extend_hint"] = wl.hint_measure(buf, torch, stream)
    if config == 2 and not args.no_others and world == 1:
        # the other batched workloads, each clocked, at full size
        line["other_configs"] = {str(c): other_config(c, args, local, torch) for c in (0, 1, 3)}
    if config == 2 and not args.no_serve and world == 1:
        # the serving loop (continuous batching over a resident genome),
        # with its own clock record
        line["serve"] = serve_phase(args, local)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
