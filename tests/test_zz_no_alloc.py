"""The allocation-free banded-DP entry point against the regular one.

esp_batch_run_band_noalloc serves callers that may not allocate device
memory once they are running (a runtime that owns every byte of device
memory through its own pool, or a request path that cannot pay for the
device-wide synchronisation cudaMalloc/cudaFree can cause).  It keeps its
scratch in one fixed device array instead.  This test runs the same batch
through the regular entry point (esp_batch_extend_device, ESP_MODE_BAND)
and twice in a row through the allocation-free one, and requires identical
results every time (the DP is integer and exact, so the tolerance is zero).
The file sorts last so that a stop-at-first-failure run has already run
every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import refgen as R  # noqa: E402
from esperanto_gb300 import _native as N  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300.extend import ExtendBuffer, ExtendParams  # noqa: E402
import workloads as W  # noqa: E402

ESP_ESCRATCH = -9


def _lib():
    L = N.lib()
    L.esp_batch_run_band_noalloc.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                             C.c_void_p, C.c_uint64,
                                             C.POINTER(N.BatchLimitsC),
                                             C.POINTER(N.ExtendParamsC), C.c_void_p,
                                             C.c_void_p, C.c_uint32, C.c_void_p]
    return L


def _batch():
    """Seeded pairs: the plain 150 x 214 workload plus shapes with N runs,
    clamped bands and m > n (the reference's own sweep shapes)."""
    arena0, pairs0 = W.synth_gotoh(5, 1536, 0)
    reads, wins, offs, halfs = [], [], [], []
    for k in range(len(pairs0)):
        r, w = B.decode_pair(arena0, pairs0[k])
        reads.append(r)
        wins.append(w)
        offs.append(32)
        halfs.append(32)
    for k, (read, win, d, off, half, _) in enumerate(R.sweep_band_block_boundaries()):
        if k % 7 == 0:
            reads.append(read)
            wins.append(win)
            offs.append(off)
            halfs.append(half)
    return B.pack_ascii_pairs(reads, wins, offs, halfs)


def _dev(a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


def test_noalloc_matches_regular_entry_point_twice():
    L = _lib()
    arena, pairs, n_iv = _batch()
    n = len(pairs)
    stride = 96
    lim = N.BatchLimitsC(int(pairs["read_len"].max()), int(pairs["win_len"].max()),
                         int(pairs["band_half"].max()))
    p = ExtendParams()._c()
    d_arena, d_pairs, d_iv = _dev(arena), _dev(pairs), _dev(n_iv)

    def outputs():
        return (torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda"),
                torch.zeros(n * stride, dtype=torch.int32, device="cuda"))

    buf = ExtendBuffer()
    ref_out, ref_cig = outputs()
    rc = L.esp_batch_extend_device(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n,
                                   d_arena.data_ptr(), arena.nbytes, d_iv.data_ptr(), len(n_iv),
                                   C.byref(lim), C.byref(p), ref_out.data_ptr(),
                                   ref_cig.data_ptr(), stride, None)
    buf.check(rc)
    torch.cuda.synchronize()
    want = ref_out.cpu().numpy().view(B.EXT_DTYPE)
    want_cig = ref_cig.cpu().numpy().reshape(n, stride)
    assert (want["status"] == 0).all()

    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out, cig = outputs()
        rc = L.esp_batch_run_band_noalloc(d_pairs.data_ptr(), n, d_arena.data_ptr(),
                                          arena.nbytes, d_iv.data_ptr(), len(n_iv),
                                          C.byref(lim), C.byref(p), out.data_ptr(),
                                          cig.data_ptr(), stride, stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(B.EXT_DTYPE)
        got_cig = cig.cpu().numpy().reshape(n, stride)
        assert np.array_equal(got, want), f"call {call}: extension records differ"
        for k in range(n):
            k_ops = int(want[k]["n_ops"])
            assert np.array_equal(got_cig[k, :k_ops], want_cig[k, :k_ops]), (call, k)


def test_noalloc_rejects_work_beyond_its_scratch():
    L = _lib()
    lim = N.BatchLimitsC(4000, 30000, -1)  # full matrices far larger than the array
    p = ExtendParams()._c()
    dummy = torch.zeros(64, dtype=torch.uint8, device="cuda")
    rc = L.esp_batch_run_band_noalloc(dummy.data_ptr(), 1, dummy.data_ptr(), 64, None, 0,
                                      C.byref(lim), C.byref(p), dummy.data_ptr(),
                                      dummy.data_ptr(), 1, None)
    assert rc == ESP_ESCRATCH


def test_noalloc_reuses_scratch_slots_and_allocates_nothing():
    """About 2,000 full-matrix pairs of ~300 x 600 bases: one block's scratch
    is ~12 MB, so the fixed array holds only five blocks and every thread
    takes several pairs from the queue in turn, reusing its scratch slot.
    Two calls in a row equal the regular entry point, and the second call
    (after the first has done the per-device set-up) leaves the device's
    free memory unchanged: no handle, no allocation."""
    L = _lib()
    rng = np.random.default_rng(9)
    reads, wins = [], []
    for k in range(2000):
        n = int(rng.integers(560, 601))
        m = int(rng.integers(260, 301))
        win = rng.choice(list("ACGT"), n)
        s = int(rng.integers(0, n - m))
        read = list(win[s:s + m])
        for q in rng.choice(m, 6, replace=False):
            read[int(q)] = str(rng.choice(list("ACGT")))
        reads.append("".join(read).encode())
        wins.append("".join(win).encode())
    arena, pairs, n_iv = B.pack_ascii_pairs(reads, wins, [0] * len(reads), [-1] * len(reads))
    n = len(pairs)
    stride = 48
    lim = N.BatchLimitsC(int(pairs["read_len"].max()), int(pairs["win_len"].max()), -1)
    p = ExtendParams()._c()
    d_arena, d_pairs = _dev(arena), _dev(pairs)
    buf = ExtendBuffer()
    ref_out = torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ref_cig = torch.zeros(n * stride, dtype=torch.int32, device="cuda")
    buf.check(L.esp_batch_extend_device(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n,
                                        d_arena.data_ptr(), arena.nbytes, None, 0, C.byref(lim),
                                        C.byref(p), ref_out.data_ptr(), ref_cig.data_ptr(),
                                        stride, None))
    torch.cuda.synchronize()
    want = ref_out.cpu().numpy().view(B.EXT_DTYPE)
    want_cig = ref_cig.cpu().numpy().reshape(n, stride)
    assert (want["status"] == 0).all()
    out = torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    cig = torch.zeros(n * stride, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out.zero_()
        cig.zero_()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.esp_batch_run_band_noalloc(d_pairs.data_ptr(), n, d_arena.data_ptr(),
                                          arena.nbytes, None, 0, C.byref(lim), C.byref(p),
                                          out.data_ptr(), cig.data_ptr(), stride, stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        got = out.cpu().numpy().view(B.EXT_DTYPE)
        got_cig = cig.cpu().numpy().reshape(n, stride)
        assert np.array_equal(got, want), f"call {call}"
        for k in range(n):
            k_ops = int(want[k]["n_ops"])
            assert np.array_equal(got_cig[k, :k_ops], want_cig[k, :k_ops]), (call, k)
