"""GPU parity at production density: every benchmark workload at (or near)
its full size through the code path the benchmark times, compared field by
field and CIGAR by CIGAR with the multi-threaded oracle -- not with another
GPU kernel.

* the 150 x 214 banded batch: all 65,536 pairs, band and extend_hint modes,
  on the one-pair kernel and on the two-pairs-per-thread kernel (all pairs
  share one geometry, so every item really holds two different pairs);
* the EA-Myers batch: all 1,048,576 pairs through the host pipeline;
* the mixed-length batch: all 4,194,304 pairs through the autotuned device
  path (length-binned paired kernel, CUDA-graph replay) and through the host
  pipeline; extend_hint on 262,144 of its pairs with the paired kernel
  forced (about 260 pairs share each hint geometry);
* split-read rescue: 16,384 reads (2.2 M flank DPs, the size at which the
  flank batch runs on the paired kernel in hint mode), with that kernel
  forced, including the DP cell census;
* the serve loop: every read of every request of a concurrent mix.

Reference semantics: extend.rs:392-428 (extend_hint), :606-1068 (run_band,
finish_extension); myers_ea.rs:249-310; split.rs:150-223, :468-570.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import ctypes as C  # noqa: E402

import oracle as O  # noqa: E402
import workloads as W  # noqa: E402
from esperanto_gb300 import _native as N  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300 import serve as SV  # noqa: E402
from esperanto_gb300 import split as S  # noqa: E402
from esperanto_gb300.extend import ExtendBuffer, ExtendParams  # noqa: E402

THREADS = os.cpu_count() or 1
STRIDE = 32

# 2-bit code byte -> its four ASCII bases (MSB first)
_LUT4 = B._ASCII[(np.arange(256)[:, None] >> (6 - 2 * np.arange(4))[None, :]) & 3]


def ascii_of(arena, n_bases):
    """ASCII bases [0, n_bases) of a 2-bit arena (4 bases per byte)."""
    nb = (n_bases + 3) // 4
    return _LUT4[arena[:nb]].reshape(-1)[:n_bases].copy()


def oracle_pairs(arena, pairs, mode, half=None):
    """The oracle over a pair batch: (cells, outputs with CIGARs)."""
    end = int(max((pairs["read_pos"] + pairs["read_len"]).max(),
                  (pairs["win_pos"] + pairs["win_len"]).max()))
    seq = ascii_of(arena, end)
    h = pairs["band_half"] if half is None else np.full(len(pairs), half, np.int32)
    return O.batch_extend(seq, pairs["read_pos"], pairs["read_len"], pairs["win_pos"],
                          pairs["win_len"], pairs["band_offset"], h, O.Params(), mode, THREADS,
                          ops_stride=STRIDE)


def assert_same(out, cig, want, mode, what):
    """Every field and every CIGAR op of a GPU batch equals the oracle's."""
    assert (out["status"] == 0).all(), (what, np.unique(out["status"]))
    for f in ("score", "read_start", "read_end", "ref_start", "n_ops"):
        bad = np.nonzero(out[f].astype(np.int64) != want[f].astype(np.int64))[0]
        assert len(bad) == 0, (what, f, bad[:8], out[f][bad[:8]], want[f][bad[:8]])
    assert int(want["n_ops"].max()) <= STRIDE, what
    used = np.arange(STRIDE)[None, :] < want["n_ops"][:, None]
    bad = np.nonzero(((cig != want["ops"]) & used).any(1))[0]
    assert len(bad) == 0, (what, "cigar", bad[:8])
    flag = out["escalated"] if mode == B.MODE_HINT else out["touched"]
    bad = np.nonzero(flag.astype(np.int32) != (want["touched"] != 0))[0]
    assert len(bad) == 0, (what, "escalated" if mode == B.MODE_HINT else "touched", bad[:8])


def test_banded_150x214_all_pairs_band_and_hint():
    arena, pairs = W.synth_gotoh(1, 65536, 0)
    for mode in (B.MODE_BAND, B.MODE_HINT):
        cells, want = oracle_pairs(arena, pairs, mode)
        for variant in (1, 3):  # one pair per thread; two pairs per thread (16x2)
            if mode == B.MODE_HINT and variant == 3:
                os.environ["ESP_GOTOH_HINT_VARIANT"] = "3"
            buf = ExtendBuffer()
            try:
                buf.set_kernel_variant(variant)
                out, cig = B.extend_batch_host(pairs, arena, mode=mode, cigar_stride=STRIDE,
                                               buf=buf)
                assert_same(out, cig, want, mode, f"banded mode {mode} variant {variant}")
                if mode == B.MODE_HINT:
                    assert B.cells_of(pairs, mode, out["escalated"]) == cells
            finally:
                os.environ.pop("ESP_GOTOH_HINT_VARIANT", None)
                buf.close()


def test_myers_all_pairs():
    arena, pairs = W.synth_myers(2, 1 << 20)
    res = B.myers_batch_host(pairs, arena)
    assert (res["status"] == 0).all()
    end = int((pairs["text_pos"] + pairs["text_len"]).max())
    seq = ascii_of(arena, end)
    cells, dist, pos = O.batch_myers_best_end(seq, pairs["read_pos"], pairs["read_len"],
                                              pairs["text_pos"], pairs["text_len"], THREADS)
    assert cells == int((pairs["read_len"].astype(np.int64) * pairs["text_len"]).sum())
    bad = np.nonzero((res["dist"] != dist) | (res["pos"].astype(np.int64) != pos))[0]
    assert len(bad) == 0, bad[:8]
    assert (dist > 30).mean() > 0.05  # the unrelated tenth is there


def test_mixed_length_all_pairs_autotuned_device_and_host():
    n = 1 << 22
    arena, pairs = W.synth_gotoh(3, n, 2)
    cells, want = oracle_pairs(arena, pairs, B.MODE_BAND)
    assert cells == B.cells_of(pairs)
    # the benchmark's device path: autotune per length class, then launches
    # replayed from a captured graph
    buf = ExtendBuffer()
    d_arena = torch.from_numpy(arena).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    d_out = torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_cig = torch.zeros(n * STRIDE, dtype=torch.int32, device="cuda")
    lim = N.BatchLimitsC(int(pairs["read_len"].max()), int(pairs["win_len"].max()),
                         int(pairs["band_half"].max()))
    p = ExtendParams()._c()
    args = (buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n, d_arena.data_ptr(), arena.nbytes,
            None, 0, C.byref(lim), C.byref(p), d_out.data_ptr(), d_cig.data_ptr(), STRIDE, None)
    variants, ms = (C.c_int * 4)(), (C.c_double * 20)()
    buf.check(N.lib().esp_batch_autotune(*args, variants, ms))
    assert any(v >= 2 for v in variants)  # the paired kernel wins at this size
    for it in range(3):  # direct, captured, replayed
        d_out.zero_()
        d_cig.zero_()
        buf.check(N.lib().esp_batch_extend_device(*args))
        torch.cuda.synchronize()
        out = d_out.cpu().numpy().view(B.EXT_DTYPE)
        cig = d_cig.cpu().numpy().view(np.uint32).reshape(n, STRIDE)
        assert_same(out, cig, want, B.MODE_BAND, f"mixed-length device run {it}")
    del d_arena, d_pairs, d_out, d_cig
    buf.close()
    # the host pipeline (two chunks on the paired kernel)
    out, cig = B.extend_batch_host(pairs, arena, cigar_stride=STRIDE, buf=ExtendBuffer())
    assert_same(out, cig, want, B.MODE_BAND, "mixed-length host pipeline")


def test_mixed_length_extend_hint_paired():
    n = 1 << 18
    arena, pairs = W.synth_gotoh(3, n, 2)
    cells, want = oracle_pairs(arena, pairs, B.MODE_HINT)
    os.environ["ESP_GOTOH_HINT_VARIANT"] = "3"
    try:
        buf = ExtendBuffer()
        out, cig = B.extend_batch_host(pairs, arena, mode=B.MODE_HINT, cigar_stride=STRIDE,
                                       buf=buf)
    finally:
        os.environ.pop("ESP_GOTOH_HINT_VARIANT", None)
    assert_same(out, cig, want, B.MODE_HINT, "mixed-length extend_hint, paired kernel")
    assert B.cells_of(pairs, B.MODE_HINT, out["escalated"]) == cells
    assert 0.05 < out["escalated"].mean() < 0.95


def test_split_reads_channel_a_paired_hint():
    n = 16384
    garena, contigs, rarena, reads, cands = W.synth_splice(4, n)
    assert 22 * len(cands) >= (1 << 20)  # the flank batch size that runs paired by default
    os.environ["ESP_GOTOH_HINT_VARIANT"] = "3"
    try:
        buf = ExtendBuffer()
        g = S.Genome(garena, contigs, buf=buf)
        out, cig, cells = S.channel_a_batch(g, reads, rarena, cands, cigar_stride=STRIDE,
                                            buf=buf)
    finally:
        os.environ.pop("ESP_GOTOH_HINT_VARIANT", None)
    assert (out["status"] == 0).all()
    ra = ascii_of(rarena, len(reads) * 150)
    found, score, ocells, d = O.batch_channel_a(garena, contigs, ra, reads["read_pos"], reads,
                                                cands, THREADS, ops_stride=STRIDE)
    assert cells == ocells  # same DP cell census: the same escalations everywhere
    assert (out["found"] == found).all()
    f = found != 0
    assert f.mean() > 0.5
    for name, got, exp in (("cand", out["cand"], d["cand"]), ("dro", out["dro"], d["dro"]),
                           ("pos", out["pos"], d["pos"]), ("score", out["score"], score),
                           ("signal", out["signal"], d["signal"]),
                           ("n_ops", out["n_ops"], d["n_ops"])):
        bad = np.nonzero((got.astype(np.int64) != exp.astype(np.int64)) & f)[0]
        assert len(bad) == 0, (name, bad[:8])
    used = (np.arange(STRIDE)[None, :] < d["n_ops"][:, None]) & f[:, None]
    assert not ((cig != d["ops"]) & used).any()


def test_serve_every_read_of_a_concurrent_mix():
    garena, contigs = W.synth_genome(5, 4_000_000, 4)
    g = S.Genome(garena, contigs)
    srv = SV.Server(g, n_streams=3, max_reads=32768, mem_budget=2 << 30)
    try:
        sizes = [800, 20000, 3000, 12000, 500, 30000, 7000, 1000, 3000]
        reqs = [W.synth_request(5, 400 + k, garena, contigs, n) for k, n in enumerate(sizes)]
        tickets = [srv.submit(a, r, STRIDE) for a, r in reqs]
        for t in tickets:
            assert srv.wait(t)[0] == 0
    finally:
        srv.destroy()
    gseq = ascii_of(garena, int(contigs["base"][-1] + contigs["len"][-1]))
    for (arena, reads), t in zip(reqs, tickets):
        pairs = SV.serve_pairs(reads, contigs)
        rseq = ascii_of(arena, len(reads) * 150)
        seq = np.concatenate([rseq, gseq])
        _, want = O.batch_extend(seq, pairs["read_pos"], pairs["read_len"],
                                 pairs["win_pos"] + len(rseq), pairs["win_len"],
                                 pairs["band_offset"], pairs["band_half"], O.Params(),
                                 B.MODE_HINT, THREADS, ops_stride=STRIDE)
        cig = t.cigar.reshape(len(reads), STRIDE)
        assert_same(t.out, cig, want, B.MODE_HINT, f"serve request of {len(reads)} reads")
