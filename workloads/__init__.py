"""Seeded synthetic workloads and GPU peak probes (BENCHMARK AND TEST TOOLING).

Not part of the alignment path: the product library
(esperanto_gb300/_lib/libesperanto_gb300.so) holds the path only, and these
build into their own libraries here:

* ``_build/libesp_synth.so`` -- synth.cpp, host-only generators of every
  benchmark workload (the reference ships no datasets; each pair draws from
  its own splitmix64 stream seeded by (seed, index), so the output does not
  depend on the thread count);
* ``_build/libesp_probe.so`` -- probe.cu, the GPU's measured integer issue
  peaks (the denominators of the DP kernels' integer roofline).

The CPU oracle's library carries a second build of synth.cpp, so the
benchmark's reference arm makes the same inputs without loading any library
of the GPU path: every generator here takes ``lib=`` to run on that build.
Declarations: workloads/esp_workloads.h.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
SYNTH_LIB = os.path.join(BUILD_DIR, "libesp_synth.so")
PROBE_LIB = os.path.join(BUILD_DIR, "libesp_probe.so")
HEADERS = [os.path.join(HERE, "esp_workloads.h"),
           os.path.join(ROOT, "include", "esperanto_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# record layouts (byte for byte the C structs of include/esperanto_gb300.h)
PAIR_DTYPE = np.dtype([("read_pos", "<u8"), ("win_pos", "<u8"), ("read_len", "<u4"),
                       ("win_len", "<u4"), ("band_offset", "<i4"), ("band_half", "<i4"),
                       ("n_first", "<u4"), ("n_read", "<u2"), ("n_win", "<u2")])
MYERS_PAIR_DTYPE = np.dtype([("read_pos", "<u8"), ("text_pos", "<u8"), ("read_len", "<u4"),
                             ("text_len", "<u4"), ("n_first", "<u4"), ("n_read", "<u2"),
                             ("n_text", "<u2")])
CONTIG_DTYPE = np.dtype([("base", "<u8"), ("len", "<u4"), ("n_first", "<u4"),
                         ("n_count", "<u4"), ("pad", "<u4")])
SPLICE_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("tail_start", "<u4"),
                              ("contig", "<u4"), ("minus", "<i4"), ("cand_first", "<u4"),
                              ("cand_count", "<u4"), ("n_first", "<u4"), ("n_read", "<u4")])
SPLICE_CAND_DTYPE = np.dtype([("contig", "<u4"), ("start", "<u4"), ("end", "<u4"),
                              ("minus_strand", "<i4"), ("support", "<u4")])
SERVE_READ_DTYPE = np.dtype([("read_pos", "<u8"), ("read_len", "<u4"), ("contig", "<u4"),
                             ("win_start", "<u4"), ("win_len", "<u4"), ("hint_offset", "<i4"),
                             ("pad", "<u4")])


class WorkloadError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} returned {code}")
        self.code = code


def _stale(lib_path, sources):
    if not os.path.exists(lib_path):
        return True
    t = os.path.getmtime(lib_path)
    return any(os.path.getmtime(f) > t for f in sources + HEADERS + [os.path.abspath(__file__)])


def build_synth(force: bool = False) -> str:
    """g++ build of the host-only generators."""
    src = os.path.join(HERE, "synth.cpp")
    if not force and not _stale(SYNTH_LIB, [src]):
        return SYNTH_LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-I", HERE,
           "-I", os.path.join(ROOT, "include"), src, "-o", SYNTH_LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


def build_probe(force: bool = False) -> str:
    """nvcc (sm_103a) build of the peak probes."""
    src = os.path.join(HERE, "probe.cu")
    if not force and not _stale(PROBE_LIB, [src]):
        return PROBE_LIB
    nvcc = next((c for c in (os.environ.get("NVCC"), shutil.which("nvcc"),
                             "/usr/local/cuda/bin/nvcc") if c and os.path.exists(c)), None)
    if nvcc is None:
        raise RuntimeError("nvcc not found: the probe library cannot be built")
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = [nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
                           "-I", HERE, "-I", os.path.join(ROOT, "include"), src,
                           "-o", PROBE_LIB + ".tmp", "-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(PROBE_LIB + ".tmp", PROBE_LIB)
    return PROBE_LIB


def build(force: bool = False):
    return build_synth(force), build_probe(force)


def bind_synth(L):
    """Set the generators' argument types on a library that exports them
    (this directory's build or the oracle's)."""
    vp, u64 = C.c_void_p, C.c_uint64
    L.esp_synth_gotoh_size.argtypes = [u64, u64, C.c_int, C.POINTER(u64)]
    L.esp_synth_gotoh.argtypes = [u64, u64, C.c_int, vp, u64, vp]
    L.esp_synth_myers_size.argtypes = [u64, u64, C.POINTER(u64)]
    L.esp_synth_myers.argtypes = [u64, u64, vp, u64, vp]
    L.esp_synth_splice_size.argtypes = [u64, u64] + [C.POINTER(u64)] * 3
    L.esp_synth_splice.argtypes = [u64, u64, vp, u64, vp, vp, u64, vp, vp, u64]
    L.esp_synth_genome.argtypes = [u64, u64, C.c_uint32, vp, u64, vp]
    L.esp_synth_serve_reads.argtypes = [u64, u64, vp, vp, C.c_uint32, u64, vp, u64, vp]
    return L


_synth = None
_probe = None


def synth_lib():
    global _synth
    if _synth is None:
        _synth = bind_synth(C.CDLL(build_synth()))
    return _synth


def probe_lib():
    global _probe
    if _probe is None:
        L = C.CDLL(build_probe())
        L.esp_probe_int_peaks.argtypes = [C.c_int] + [C.POINTER(C.c_double)] * 4
        L.esp_probe_simd16_peaks.argtypes = [C.c_int] + [C.POINTER(C.c_double)] * 2
        _probe = L
    return _probe


def _check(rc, what):
    if rc:
        raise WorkloadError(rc, what)


def synth_gotoh(seed: int, n_pairs: int, shape: int, lib=None):
    """Gotoh workload, shape 0 (150-bp reads vs 214-bp windows, half 32 at
    offset 32) or 2 (mixed length): (arena, pairs)."""
    L = lib or synth_lib()
    nb = C.c_uint64()
    _check(L.esp_synth_gotoh_size(seed, n_pairs, shape, C.byref(nb)), "esp_synth_gotoh_size")
    arena = np.zeros(nb.value, np.uint8)
    pairs = np.zeros(n_pairs, PAIR_DTYPE)
    _check(L.esp_synth_gotoh(seed, n_pairs, shape, arena.ctypes.data, nb.value,
                             pairs.ctypes.data), "esp_synth_gotoh")
    return arena, pairs


def synth_myers(seed: int, n_pairs: int, lib=None):
    """Myers workload (150-bp queries vs 200-bp texts): (arena, myers pairs)."""
    L = lib or synth_lib()
    nb = C.c_uint64()
    _check(L.esp_synth_myers_size(seed, n_pairs, C.byref(nb)), "esp_synth_myers_size")
    arena = np.zeros(nb.value, np.uint8)
    pairs = np.zeros(n_pairs, MYERS_PAIR_DTYPE)
    _check(L.esp_synth_myers(seed, n_pairs, arena.ctypes.data, nb.value, pairs.ctypes.data),
           "esp_synth_myers")
    return arena, pairs


def synth_splice(seed: int, n_reads: int, lib=None):
    """Split-read rescue workload: (genome_arena, contigs, read_arena, reads,
    cands)."""
    L = lib or synth_lib()
    gb, rb, nc = C.c_uint64(), C.c_uint64(), C.c_uint64()
    _check(L.esp_synth_splice_size(seed, n_reads, C.byref(gb), C.byref(rb), C.byref(nc)),
           "esp_synth_splice_size")
    garena = np.zeros(gb.value, np.uint8)
    contigs = np.zeros(n_reads, CONTIG_DTYPE)
    rarena = np.zeros(rb.value, np.uint8)
    reads = np.zeros(n_reads, SPLICE_READ_DTYPE)
    cands = np.zeros(nc.value, SPLICE_CAND_DTYPE)
    _check(L.esp_synth_splice(seed, n_reads, garena.ctypes.data, gb.value, contigs.ctypes.data,
                              rarena.ctypes.data, rb.value, reads.ctypes.data,
                              cands.ctypes.data, nc.value), "esp_synth_splice")
    return garena, contigs, rarena, reads, cands


def synth_genome(seed: int, total_bases: int, n_contigs: int, lib=None):
    """Uniform-ACGT genome: (arena, contigs)."""
    L = lib or synth_lib()
    stride = ((total_bases + n_contigs - 1) // n_contigs + 3) // 4 * 4
    arena = np.zeros(stride * n_contigs // 4 + 16, np.uint8)
    contigs = np.zeros(n_contigs, CONTIG_DTYPE)
    _check(L.esp_synth_genome(seed, total_bases, n_contigs, arena.ctypes.data, len(arena),
                              contigs.ctypes.data), "esp_synth_genome")
    return arena, contigs


def synth_request(seed: int, request: int, genome_arena: np.ndarray, contigs: np.ndarray,
                  n_reads: int, lib=None):
    """Paired-end serve request reads: (read arena, serve reads)."""
    L = lib or synth_lib()
    arena = np.zeros((n_reads * 150 + 3) // 4 + 16, np.uint8)
    reads = np.zeros(n_reads, SERVE_READ_DTYPE)
    _check(L.esp_synth_serve_reads(seed, request, genome_arena.ctypes.data, contigs.ctypes.data,
                                   len(contigs), n_reads, arena.ctypes.data, len(arena),
                                   reads.ctypes.data), "esp_synth_serve_reads")
    return arena, reads


def int_peaks(device: int = 0):
    """(lop3, imnmx, iadd, imad) lane-ops/s measured on `device`."""
    v = [C.c_double() for _ in range(4)]
    _check(probe_lib().esp_probe_int_peaks(device, *[C.byref(x) for x in v]),
           "esp_probe_int_peaks")
    return tuple(x.value for x in v)


def simd16_peaks(device: int = 0):
    """(add-max, 3-way max) 16x2 lane-ops/s measured on `device`."""
    v = [C.c_double() for _ in range(2)]
    _check(probe_lib().esp_probe_simd16_peaks(device, *[C.byref(x) for x in v]),
           "esp_probe_simd16_peaks")
    return tuple(x.value for x in v)


def declared_symbols():
    """Names declared in esp_workloads.h (for the load test)."""
    import re
    with open(os.path.join(HERE, "esp_workloads.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:[\w ]+\*?\s*)\b(esp_\w+)\s*\(", text, re.M)))
