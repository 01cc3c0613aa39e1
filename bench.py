"""Benchmark: batched banded Gotoh with traceback on one GB300 (or N replicas).

Default workload = the mixed-length batched configuration: 4,194,304 read x
window pairs, read length U[50,300], band half-width in {16,32,64,128} w.p.
{.4,.3,.2,.1}, windows of read + 2*half, full CIGAR traceback (seeded
synthetic data; the reference ships no dataset).  One step = one pass of the
DP over the whole batch.  Metric: GCUPS (DP cells = sum over rows of the
in-window width, crates/map/src/extend.rs:653-696).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--config 0|2] [--pairs P]

Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
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

OPS_PER_CELL = 21  # integer ops of the cell recurrence as written in gotoh.cu (see DESIGN)
INT_LANES_PER_SM = 128
# Myers: 10 32-bit ops per 32-cell limb per text column (wide-word step)
MYERS_OPS_PER_CELL = 10.0 / 32.0


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def workload_desc(config: int, n: int) -> str:
    if config == 1:
        return (f"bit-parallel EA-Myers infix_best_end: {n} pairs, 150-bp query vs 200-bp "
                "text, 0-8 edits, 10% unrelated")
    if config == 0:
        return (f"plain banded Gotoh: {n} pairs, 150-bp reads vs 214-bp windows, "
                "band half 32 at offset 32, traceback to CIGAR")
    return (f"batched uneven Gotoh: {n} pairs, read U[50,300], half {{16,32,64,128}} "
            "w.p. {.4,.3,.2,.1}, window read+2*half, traceback to CIGAR")


class ClockSampler:
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


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gpu" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def ascii_of_prefix(arena, pairs):
    from esperanto_gb300 import batch as B
    end = int((pairs["win_pos"] + pairs["win_len"]).max())
    return B._ASCII[B.unpack_codes(arena, 0, end)]


def cpu_reference(args, config, n_pairs, seed, threads):
    """The reference's CPU path (restated scalar kernel) on a bounded sample."""
    import oracle as O
    from esperanto_gb300 import batch as B
    sample = args.cpu_sample
    if config == 1:
        sample = sample * 16
        arena, pairs = B.synth_myers(seed, sample)
        end = int((pairs["text_pos"] + pairs["text_len"]).max())
        seq = B._ASCII[B.unpack_codes(arena, 0, end)]
        O.build()

        def run_m():
            t = time.perf_counter()
            cells, _, _ = O.batch_myers_best_end(seq, pairs["read_pos"], pairs["read_len"],
                                                 pairs["text_pos"], pairs["text_len"], threads)
            return cells, time.perf_counter() - t
        return run_m, sample
    arena, pairs = B.synth_gotoh(seed, sample, config)
    seq = ascii_of_prefix(arena, pairs)
    O.build()

    def run():
        t = time.perf_counter()
        cells, _ = O.batch_extend(seq, pairs["read_pos"], pairs["read_len"], pairs["win_pos"],
                                  pairs["win_len"], pairs["band_offset"], pairs["band_half"],
                                  O.Params(), 0, threads)
        return cells, time.perf_counter() - t
    return run, sample


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[0, 1, 2])
    ap.add_argument("--pairs", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_init(args)
    config = args.config
    n_pairs = args.pairs or {0: 65536, 1: 1048576, 2: 4194304}[config]
    seed = {0: 1, 1: 2, 2: 3}[config] + 1000 * rank  # weak scaling: each rank its own batch
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        run, sample = cpu_reference(args, config, n_pairs, seed, threads)
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
                "scaling": "weak", "vs_baseline": None,
                "dtype": "u32" if config == 1 else "int16",
                "data": "synthetic", "config": {"workload": workload_desc(config, sample),
                                                 "sample_of": n_pairs},
                "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                                 "sample": f"{sample} pairs of the workload per step"},
                "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    from esperanto_gb300 import _native as N
    from esperanto_gb300 import batch as B
    from esperanto_gb300.extend import ExtendBuffer, ExtendParams
    import ctypes as C

    buf = ExtendBuffer(local)
    stride = 32
    L = N.lib()
    stream = torch.cuda.ExternalStream(buf.stream_ptr())
    p = ExtendParams()._c()
    if config == 1:
        arena, pairs = B.synth_myers(seed, n_pairs)
        cells = int((pairs["read_len"].astype(np.int64) * pairs["text_len"]).sum())
        res_dtype = B.MYERS_RES_DTYPE
    else:
        arena, pairs = B.synth_gotoh(seed, n_pairs, config)
        cells = B.cells_of(pairs)
        res_dtype = B.EXT_DTYPE
    d_arena = torch.from_numpy(arena).to(f"cuda:{local}")
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).to(f"cuda:{local}")
    d_out = torch.empty(n_pairs * res_dtype.itemsize, dtype=torch.uint8, device=f"cuda:{local}")
    d_cig = torch.empty(max(1, n_pairs * stride if config != 1 else 1), dtype=torch.int32,
                        device=f"cuda:{local}")
    if config == 1:
        def step():
            rc = L.esp_batch_myers_device(buf.handle, B.MYERS_BEST_END, d_pairs.data_ptr(),
                                          n_pairs, 150, d_arena.data_ptr(), arena.nbytes, None,
                                          0, d_out.data_ptr(), None)
            buf.check(rc)
    else:
        lim = N.BatchLimitsC(int(pairs["read_len"].max()), int(pairs["win_len"].max()),
                             int(pairs["band_half"].max()))

        def step():
            rc = L.esp_batch_extend_device(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n_pairs,
                                           d_arena.data_ptr(), arena.nbytes, None, 0,
                                           C.byref(lim), C.byref(p), d_out.data_ptr(),
                                           d_cig.data_ptr(), stride, None)
            buf.check(rc)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    out_host = d_out.cpu().numpy().view(res_dtype)
    bad = int((out_host["status"] != 0).sum())
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with torch.cuda.stream(stream):
        evs[0].record(stream)
        for k in range(args.steps):
            step()
            evs[k + 1].record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop(local)
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = sum(per_step) / args.steps
    launches = int(L.esp_last_launch_count(buf.handle)) * args.steps
    tmax = torch.tensor([ms], dtype=torch.float64, device=f"cuda:{local}")
    tcells = torch.tensor([float(cells)], dtype=torch.float64, device=f"cuda:{local}")
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(tcells, op=dist.ReduceOp.SUM)
    ms_max = float(tmax.item())
    value = float(tcells.item()) / (ms_max / 1e3) / 1e9

    # end to end: host arrays (pinned) through the host C-ABI call
    pin_arena = torch.from_numpy(arena).pin_memory().numpy()
    pin_pairs = torch.from_numpy(pairs.view(np.uint8)).pin_memory().numpy()
    out_pin = torch.empty(n_pairs * res_dtype.itemsize, dtype=torch.uint8).pin_memory().numpy()
    cig_pin = torch.empty(n_pairs * stride if config != 1 else 1,
                          dtype=torch.int32).pin_memory().numpy()

    def e2e_step():
        if config == 1:
            rc = L.esp_batch_myers_host(buf.handle, B.MYERS_BEST_END, pin_pairs.ctypes.data,
                                        n_pairs, pin_arena.ctypes.data, pin_arena.nbytes, None,
                                        0, out_pin.ctypes.data)
        else:
            rc = L.esp_batch_extend_host(buf.handle, B.MODE_BAND, pin_pairs.ctypes.data,
                                         n_pairs, pin_arena.ctypes.data, pin_arena.nbytes,
                                         None, 0, C.byref(p), out_pin.ctypes.data,
                                         cig_pin.ctypes.data, stride)
        buf.check(rc)
    e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_val = cells / e2e_s / 1e9
    h2d = pin_arena.nbytes + pin_pairs.nbytes
    d2h = out_pin.nbytes + (cig_pin.nbytes if config != 1 else 0)

    if rank != 0:
        return
    peaks, src = load_peaks()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    peak_ops = sm_count * INT_LANES_PER_SM * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    ops_per_cell = MYERS_OPS_PER_CELL if config == 1 else OPS_PER_CELL
    achieved_ops = cells * ops_per_cell / (ms / 1e3) / 1e12
    cpu = None
    if not args.no_cpu_baseline:
        run, sample = cpu_reference(args, config, n_pairs, seed, threads)
        run()
        c, dt = run()
        cpu = {"value": c / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
               "sample": f"{sample} pairs of the same workload, restated scalar kernel "
                         f"(run_band<i16>, what the reference runs on aarch64)"}
    line = {
        "metric": "GCUPS", "value": value, "unit": "GCUPS", "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32" if config == 1 else "int16", "data": "synthetic",
        "config": {"workload": workload_desc(config, n_pairs), "pairs": n_pairs,
                   "cells_per_step": cells,
                   "mode": "myers_ea::long::infix_best_end" if config == 1 else "run_band",
                   "l2": "inputs larger than L2 (arena %.0f MB + traceback scratch)"
                         % (arena.nbytes / 1e6)},
        "pairs_per_s": n_pairs * world / (ms_max / 1e3),
        "bad_status": bad,
        "gpu_launches": launches,
        "roofline": {"bound": "int_alu", "achieved": achieved_ops, "peak": peak_ops,
                     "unit": "Tops/s", "frac": achieved_ops / peak_ops, "traffic": None,
                     "peak_source": f"nominal: {sm_count} SMs x {INT_LANES_PER_SM} INT32 lanes x "
                                    f"{peaks.get('sm_max_mhz', 2070.0):.0f} MHz ({src} clock)",
                     "ops_per_cell": ops_per_cell},
        "e2e": {"value": e2e_val, "unit": "GCUPS", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "per_step_ms": per_step,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
