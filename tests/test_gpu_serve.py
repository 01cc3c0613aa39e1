"""The serving loop: results are identical alone and in a concurrent mix,
match the batch API and the oracle, and admission / closing behave."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import oracle as O  # noqa: E402
from esperanto_gb300 import EspError  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300 import serve as SV  # noqa: E402
from esperanto_gb300.split import Genome  # noqa: E402
import workloads as W  # noqa: E402


@pytest.fixture(scope="module")
def setup():
    garena, contigs = W.synth_genome(5, 4_000_000, 4)
    g = Genome(garena, contigs)
    srv = SV.Server(g, n_streams=3, max_reads=32768, mem_budget=2 << 30)
    yield garena, contigs, g, srv
    srv.destroy()


def _key(t, k):
    o = t.out[k]
    return (int(o["score"]), int(o["read_start"]), int(o["read_end"]), int(o["ref_start"]),
            tuple(B.cigar_of(t.cigar.reshape(len(t.reads), t.stride)[k], int(o["n_ops"]))))


def test_alone_equals_mix_equals_batch_and_oracle(setup):
    garena, contigs, g, srv = setup
    arena, reads = W.synth_request(5, 1, garena, contigs, 3000)
    alone = srv.submit(arena, reads)
    st, lat = srv.wait(alone)
    assert st == 0 and lat > 0
    ref = [_key(alone, k) for k in range(len(reads))]
    # the same request in a mix of concurrent requests of other sizes
    mix = []
    for k, n in enumerate([800, 20000, 3000, 12000, 500, 30000, 7000, 1000]):
        a2, r2 = W.synth_request(5, 100 + k, garena, contigs, n)
        mix.append(srv.submit(a2, r2))
        if k == 3:
            again = srv.submit(arena, reads)
    for t in mix + [again]:
        assert srv.wait(t)[0] == 0
    assert [_key(again, k) for k in range(len(reads))] == ref
    # the batch API on the same pairs (windows read from a genome copy)
    pairs = SV.serve_pairs(reads, contigs)
    read_bits = B.unpack_codes(arena, 0, len(reads) * 150)
    gb = B.unpack_codes(garena, 0, int(contigs["base"][-1] + contigs["len"][-1]))
    codes = np.concatenate([read_bits, gb])
    comb = B.pack_codes(codes)
    pairs2 = pairs.copy()
    pairs2["win_pos"] = pairs["win_pos"] + len(reads) * 150
    out, cig = B.extend_batch_host(pairs2, comb, mode=B.MODE_HINT, cigar_stride=32)
    for k in range(len(reads)):
        o = out[k]
        assert (int(o["score"]), int(o["read_start"]), int(o["read_end"]), int(o["ref_start"]),
                tuple(B.cigar_of(cig[k], int(o["n_ops"])))) == ref[k]
    # the oracle on a sample
    for k in range(0, len(reads), 97):
        r = B._ASCII[read_bits[k * 150:(k + 1) * 150]].tobytes()
        ws, wl = int(pairs["win_pos"][k]), int(pairs["win_len"][k])
        w = B._ASCII[gb[ws:ws + wl]].tobytes()
        assert O.extend_hint(r, w, O.Params(), offset=int(pairs["band_offset"][k])).key() == ref[k]


def _keys(t):
    return [_key(t, k) for k in range(len(t.reads))]


def test_large_requests_split_small_ones_share_launches(setup):
    """A request of 60,000 reads on a server of 8,192-read launches runs
    over several launches; ten small requests queued behind it share a
    launch with its tail; every result equals the request run alone on the
    module's server."""
    garena, contigs, g, srv = setup
    big = W.synth_request(5, 7, garena, contigs, 60000)
    small = [W.synth_request(5, 500 + k, garena, contigs, 300 + 50 * k) for k in range(10)]
    want = []
    for a, r in [big] + small:
        t = srv.submit(a, r)
        assert srv.wait(t)[0] == 0
        want.append(_keys(t))
    s1 = SV.Server(g, n_streams=1, max_reads=8192, mem_budget=1 << 30)
    try:
        ts = [s1.submit(a, r) for a, r in [big] + small]
        for t in ts:
            assert s1.wait(t)[0] == 0
        assert [_keys(t) for t in ts] == want
        st = s1.stats()
        assert st["split_requests"] >= 1 and st["merged_launches"] >= 1, st
        assert st["reads"] == sum(len(r) for _, r in [big] + small)
        assert st["launches"] >= 8
    finally:
        s1.destroy()


def test_memory_budget_binds_before_slots(setup):
    """Four slots but scratch for about one and a half launches: the second
    launch is cut to the scratch left, later requests wait at the head of
    the queue for scratch (not for a slot) and run when a launch returns its
    share; the pool is never over-committed and every result equals the
    ample-budget server's."""
    garena, contigs, g, srv = setup
    reqs = [W.synth_request(5, 600 + k, garena, contigs, 8192) for k in range(6)]
    want = []
    for a, r in reqs:
        t = srv.submit(a, r)
        assert srv.wait(t)[0] == 0
        want.append(_keys(t))
    # one 8,192-read launch of 150 x 214 extend_hint pairs charges 256 warps
    # x 4,280 words x 32 lanes x 4 bytes = 140 MB
    budget = 210 << 20
    s2 = SV.Server(g, n_streams=4, max_reads=8192, mem_budget=budget)
    try:
        ts = [s2.submit(a, r) for a, r in reqs]
        for t in ts:
            assert s2.wait(t)[0] == 0
        assert [_keys(t) for t in ts] == want
        st = s2.stats()
        assert st["budget_waits"] >= 1 and st["cut_launches"] >= 1, st
        assert st["pool_bytes"] <= budget and st["pool_peak_bytes"] <= st["pool_bytes"], st
        assert st["pool_peak_bytes"] > (140 << 20), st
    finally:
        s2.destroy()
    # a request whose smallest launch cannot fit the budget is refused
    s3 = SV.Server(g, n_streams=2, max_reads=8192, mem_budget=8 << 20)
    try:
        with pytest.raises(EspError) as ei:
            s3.submit(*reqs[0])
        assert ei.value.code == -6  # ESP_EBUSY
    finally:
        s3.destroy()


def test_bounded_wait_times_out_then_completes(setup):
    """esp_server_wait with a zero timeout on a request still in flight
    returns ESP_ETIMEOUT and keeps the ticket; a later wait collects it."""
    garena, contigs, g, srv = setup
    t = srv.submit(*W.synth_request(5, 9, garena, contigs, 60000))
    with pytest.raises(EspError) as ei:
        srv.wait(t, 0)
    assert ei.value.code == -7  # ESP_ETIMEOUT
    st, lat = srv.wait(t, 60000)
    assert st == 0 and lat > 0
    # an empty request completes at once
    a, r = W.synth_request(5, 10, garena, contigs, 10)
    assert srv.wait(srv.submit(a, r[:0]), 1000)[0] == 0


def test_admission_and_close(setup):
    garena, contigs, g, srv = setup
    srv2 = SV.Server(g, n_streams=1, max_reads=32768, mem_budget=1 << 30)
    # requests are built first so that all six are queued within microseconds
    # and the single slot is still busy with the first when close() lands
    reqs = [W.synth_request(5, 200 + k, garena, contigs, 30000) for k in range(6)]
    ts = [srv2.submit(*r) for r in reqs]
    srv2.close()
    sts = [srv2.wait(t)[0] for t in ts]
    assert sts[0] == 0                      # already admitted: finishes normally
    assert any(s == -8 for s in sts[1:])    # still queued at close: ESP_ECLOSED
    with pytest.raises(EspError):
        srv2.submit(*W.synth_request(5, 300, garena, contigs, 100))
    srv2.destroy()
