"""GPU parity for the Gotoh DP: the sm_103a kernels against the reference's
known answers and against the oracle on the reference's seeded sweeps."""
import numpy as np
import pytest

import oracle as O
import refgen as R
from golden_check import check_extension, load

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import esperanto_gb300 as E  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from gpu_helpers import _compare, compare, gpu_batch, kernel_buffer  # noqa: E402
import workloads as W  # noqa: E402


def _gpu_kind(kind, case):
    p = E.ExtendParams(**case["params"])
    band = tuple(case["band"]) if case.get("band") is not None else None
    r, w = case["read"], case["window"]
    if kind in ("run_band_i16", "run_band_i32", "run_dispatch"):
        return E.run_band(r, w, p, band=band)[0]
    if kind == "extend":
        return E.extend(r, w, p)
    if kind == "extend_hint":
        return E.extend_hint(r, w, p, hint=E.DiagHint(case.get("offset", 0)))
    raise AssertionError(kind)


def test_known_answers_per_call():
    G = load()
    for case in G["extension"]:
        for kind in case["kinds"]:
            check_extension(_gpu_kind(kind, case), case["expect"], f"{case['name']} [{kind}]")


def test_sweep_band_block_boundaries():
    cases, dirs, ctx = [], [], []
    for read, win, d, off, half, c in R.sweep_band_block_boundaries():
        cases.append((read, win, (off, half)))
        dirs.append(d)
        ctx.append(c)
    assert compare(cases, dirs, ctxs=ctx) > 3000


def test_sweep_band():
    cases, dirs, ctx = [], [], []
    for read, win, d, off, half, c in R.sweep_band():
        if len(win) > 2000:
            continue  # long windows run in their own test
        cases.append((read, win, (off, half)))
        dirs.append(d)
        ctx.append(c)
    assert compare(cases, dirs, ctxs=ctx) > 400


def test_sweep_full_block_boundaries():
    cases, dirs, ctx = [], [], []
    for read, win, d, c in R.sweep_full_block_boundaries():
        cases.append((read, win, None))
        dirs.append(d)
        ctx.append(c)
    compare(cases, dirs, ctxs=ctx)


def test_sweep_full_matrix():
    cases, dirs, ctx = [], [], []
    for read, win, d, c in R.sweep_full_matrix():
        if len(win) > 3000:
            continue
        cases.append((read, win, None))
        dirs.append(d)
        ctx.append(c)
    assert compare(cases, dirs, ctxs=ctx) > 300


def test_long_windows_20000():
    # n = 20,000 (the documented maximum window, extend.rs:2612-2622, :2793-2821)
    cases, dirs = [], []
    for read, win, d, c in R.sweep_full_matrix():
        if len(win) == 20000:
            cases.append((read, win, None))
            dirs.append(d)
    for read, win, d, off, half, c in R.sweep_band():
        if len(win) == 20000:
            cases.append((read, win, (off, half)))
            dirs.append(d)
    compare(cases, dirs)


def test_hint_policy_sweep():
    rng = R.Rng(0x5151)
    cases, dirs = [], []
    for m, n in [(8, 9), (20, 29), (20, 31), (60, 120), (150, 214), (150, 400), (100, 30)]:
        for rep in range(6):
            read = R.rand_seq(rng, m)
            win = R.rand_window(rng, read, n) if rep % 2 == 0 else R.rand_seq(rng, n)
            off = rng.below(n + 20) - 10
            cases.append((read, win, (off, 30)))
            dirs.append(rep % 3)
    compare(cases, dirs, mode=B.MODE_HINT)


def test_banded_150x214_subset_band_and_hint():
    arena, pairs = W.synth_gotoh(1, 2048, 0)
    cases = []
    for k in range(len(pairs)):
        r, w = B.decode_pair(arena, pairs[k])
        cases.append((r, w, (int(pairs[k]["band_offset"]), int(pairs[k]["band_half"]))))
    compare(cases, [0] * len(cases))
    compare(cases, [0] * len(cases), mode=B.MODE_HINT)


def test_mixed_length_subset():
    arena, pairs = W.synth_gotoh(3, 1024, 2)
    cases = []
    for k in range(len(pairs)):
        r, w = B.decode_pair(arena, pairs[k])
        cases.append((r, w, (int(pairs[k]["band_offset"]), int(pairs[k]["band_half"]))))
    compare(cases, [1] * len(cases))


def test_batch_direct_synth_matches_oracle_batch():
    # the synthetic arena straight into the batch API (no ASCII round trip)
    arena, pairs = W.synth_gotoh(11, 4096, 0)
    out, cig = B.extend_batch_host(pairs, arena, params=E.ExtendParams(), mode=B.MODE_BAND,
                                   cigar_stride=32)
    assert (out["status"] == 0).all()
    for k in range(0, len(pairs), 97):
        r, w = B.decode_pair(arena, pairs[k])
        want = O.run_dispatch(r, w, O.Params(), band=(32, 32))[0].key()
        got = (int(out[k]["score"]), int(out[k]["read_start"]), int(out[k]["read_end"]),
               int(out[k]["ref_start"]), tuple(B.cigar_of(cig[k], int(out[k]["n_ops"]))))
        assert got == want


def test_empty_and_degenerate_inputs():
    assert E.run_band(b"", b"ACGT")[0].key() == (0, 0, 0, 0, ())
    assert E.run_band(b"ACGT", b"")[0].key() == (0, 0, 0, 0, (("S", 4),))
    assert E.extend_hint(b"ACGT", b"").key() == (0, 0, 0, 0, (("S", 4),))
    # all-N read: score 0, whole-read soft clip
    assert E.extend(b"NNNN", b"ACGT").key() == O.extend(b"NNNN", b"ACGT").key()


def test_cigar_capacity_reported():
    read = b"ACGT" * 10
    win = b"ACGA" * 10
    with pytest.raises(E.EspError):
        import ctypes as C
        from esperanto_gb300 import _native as N
        buf = E.extend._default_buffer() if hasattr(E.extend, "_default_buffer") else None
        from esperanto_gb300.extend import _default_buffer
        buf = _default_buffer()
        p = E.ExtendParams()._c()
        out = N.ExtensionC()
        ops = (C.c_uint32 * 1)()
        rc = N.lib().esp_extend(buf.handle, read, len(read), win, len(win), C.byref(p),
                                C.byref(out), ops, 1)
        buf.check(rc)


def _long_pair(rng, m, n, indels=True):
    """A read of m bases planted in a window of n with substitutions and,
    when asked, a few short indels."""
    win = rng.choice(list("ACGT"), n)
    s = int(rng.integers(0, max(1, n - m)))
    read = list(win[s:s + m]) + list(rng.choice(list("ACGT"), max(0, m - (n - s))))
    for q in rng.choice(m, m // 200 + 1, replace=False):
        read[int(q)] = str(rng.choice(list("ACGT")))
    if indels:
        for q in sorted(rng.choice(np.arange(10, m - 10), 4, replace=False), reverse=True):
            if rng.random() < 0.5:
                read.pop(int(q))
                read.append("A")
            else:
                read.insert(int(q), "C")
                read.pop()
    return "".join(read[:m]).encode(), "".join(win).encode(), s


def test_wide_reads_match_the_i32_flavour():
    """Reads whose scores leave the int16 row buffer (longer than 8191 /
    largest substitution score: 4,095 bases at the default +2 match) run in
    the int32 wide kernel instead of being refused, and return what the
    reference's i32 flavour of run_band returns (extend.rs:462-528), up to
    20,000-base reads with scores above 32,767: per call and in batches
    mixed with int16-domain pairs, band and full matrix, every EditDir."""
    rng = np.random.default_rng(77)
    cases = []  # (read, win, band or None, edit_dir)
    for m, n, band in ((4095, 4200, (2, 40)), (4096, 4200, (2, 40)), (5000, 5100, None),
                       (8191, 8300, (30, 64)), (12000, 12100, (40, 30)),
                       (20000, 20000, (0, 30)), (20000, 20050, (10, 128)), (6000, 6000, None)):
        read, win, s = _long_pair(rng, m, n)
        off = band[0] if band else 0
        cases.append((read, win, (s + off, band[1]) if band else None, len(cases) % 3))
    for read, win, band, d in cases:
        want, wt = O.run_band(read, win, O.Params(edit_dir=d), wide=True, band=band)
        got, gt = E.run_band(read, win, E.ExtendParams(edit_dir=d), band=band)
        assert got.key() == want.key(), (len(read), band, d)
        assert (gt.touched, gt.row, gt.left) == (wt.touched, wt.row, wt.left)
    assert max(O.run_band(c[0], c[1], wide=True, band=c[2])[0].score for c in cases) > 32767
    # extend_hint on long reads (both attempts in the wide kernel)
    for read, win, band, d in cases[:5]:
        want = O.extend_hint(read, win, O.Params(edit_dir=d), offset=band[0] if band else 0,
                             wide=True)
        got = E.extend_hint(read, win, E.ExtendParams(edit_dir=d),
                            hint=E.DiagHint(band[0] if band else 0))
        assert got.key() == want.key(), (len(read), d)
    # batches: long pairs among 150 x 214 pairs, on every DP kernel, band and hint
    short = []
    for k in range(300):
        read, win, s = _long_pair(rng, 150, 214, indels=k % 2 == 0)
        short.append((read, win, (s, 32)))
    mixed = short[:150] + [(c[0], c[1], c[2]) for c in cases[:6]] + short[150:]
    for kern in ("warp", "thread", "paired"):
        for mode in (B.MODE_BAND, B.MODE_HINT):
            got = gpu_batch(mixed, 0, mode, cigar_stride=64, kernel=kern)
            for k, (read, win, band) in enumerate(mixed):
                if mode == B.MODE_BAND:
                    want = O.run_band(read, win, O.Params(), wide=True, band=band)[0].key()
                else:
                    want = O.extend_hint(read, win, O.Params(), offset=band[0] if band else 0,
                                         wide=True).key()
                assert got[k][0] == want, (kern, mode, k, len(read))


def test_graph_replay_of_identical_device_batches():
    """Identical device submissions are captured once and replayed as a CUDA
    graph; replays read the buffers' current contents, so alternating inputs
    through the same buffers gives each input's own results."""
    import ctypes as C
    from esperanto_gb300 import _native as N
    from esperanto_gb300.extend import ExtendBuffer, ExtendParams
    n = 20000  # above the warp-per-pair size: binning + persistent kernel
    sets = [W.synth_gotoh(s, n, 2) for s in (11, 12)]
    size = max(a.nbytes for a, _ in sets)
    lim = N.BatchLimitsC(300, 300 + 256, 128)
    p = ExtendParams()._c()
    buf = ExtendBuffer()
    d_arena = torch.zeros(size + 64, dtype=torch.uint8, device="cuda")
    d_pairs = torch.zeros(n * B.PAIR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_cig = torch.zeros(n * 32, dtype=torch.int32, device="cuda")
    want = [B.extend_batch_host(pr, ar, cigar_stride=32) for ar, pr in sets]
    for it in range(6):
        ar, pr = sets[it % 2]
        d_arena[:ar.nbytes].copy_(torch.from_numpy(ar))
        d_pairs.copy_(torch.from_numpy(pr.view(np.uint8)))
        torch.cuda.synchronize()
        rc = N.lib().esp_batch_extend_device(buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n,
                                             d_arena.data_ptr(), size, None, 0, C.byref(lim),
                                             C.byref(p), d_out.data_ptr(), d_cig.data_ptr(), 32,
                                             None)
        buf.check(rc)
        torch.cuda.synchronize()
        out = d_out.cpu().numpy().view(B.EXT_DTYPE)
        cig = d_cig.cpu().numpy().view(np.uint32).reshape(n, 32)
        wo, wc = want[it % 2]
        assert (out == wo).all()
        for k in range(0, n, 97):
            assert (cig[k, :out[k]["n_ops"]] == wc[k, :out[k]["n_ops"]]).all()


def _geometry_groups(seed, groups, per_group):
    """Cases in groups of one band geometry (read length, window length,
    offset, half): what the paired kernel runs two to a thread.  Reads are
    mutated window slices; some reads and some windows carry N."""
    rng = np.random.default_rng(seed)
    cases, ctx = [], []
    for gi, (m, n, off, half) in enumerate(groups):
        for k in range(per_group):
            win = rng.choice(list("ACGT"), n)
            s = int(rng.integers(0, max(1, n - m + 1)))
            read = list(win[s:s + m]) + list(rng.choice(list("ACGT"), max(0, m - (n - s))))
            read = read[:m]
            for _ in range(int(rng.integers(0, 6))):  # substitutions, indels
                if not read:
                    break
                q = int(rng.integers(0, len(read)))
                kind = int(rng.integers(0, 3))
                if kind == 0:
                    read[q] = str(rng.choice(list("ACGT")))
                elif kind == 1:
                    read.insert(q, str(rng.choice(list("ACGT"))))
                    read.pop()
                else:
                    read.pop(q)
                    read.append(str(rng.choice(list("ACGT"))))
            if k % 7 == 3 and m > 2:
                read[m // 2] = "N"
            if k % 5 == 1:  # a window N: this pair runs alone
                win[n // 3] = "N"
            cases.append(("".join(read).encode(), "".join(win).encode(),
                          (off, half) if half >= 0 else None))
            ctx.append(f"group {gi} {(m, n, off, half)} pair {k}")
    return cases, ctx


def test_paired_kernel_geometry_groups():
    """Two pairs per thread (16x2 lanes): groups of identical geometry --
    single strips, ragged last strips, clamped band edges, full matrices --
    with odd group sizes so some neighbours differ and run one after the
    other; every pair matches the oracle."""
    groups = [(1, 5, 0, 2), (7, 20, 3, 4), (8, 40, 2, 16), (9, 60, 16, 16), (31, 95, 32, 32),
              (150, 214, 32, 32), (150, 150, -20, 16), (64, 300, 250, 8), (301, 301, 0, 64),
              (40, 50, 0, -1), (17, 33, 0, -1), (100, 230, 65, 64), (250, 510, 128, 128)]
    cases, ctx = _geometry_groups(5, groups, 37)
    dirs = [k % 3 for k in range(len(cases))]
    assert compare(cases, dirs, ctxs=ctx, kernels=("paired",)) == len(cases)
    # extend_hint batches on a handle set to a paired variant run the
    # one-pair kernel (hint offsets differ per pair) with the same results
    hint = [(r, w, (band[0] if band else 0, 30)) for r, w, band in cases[:200]]
    assert _compare(hint, dirs[:200], B.MODE_HINT, None, "paired") == 200


def test_paired_kernel_variants_on_mixed_batch():
    """Both paired variants (3 and 4 blocks per SM) on the mixed-length
    workload equal the one-pair kernel bit for bit (results and CIGARs)."""
    from esperanto_gb300.extend import ExtendBuffer
    ar, pr = W.synth_gotoh(31, 50000, 2)
    want = B.extend_batch_host(pr, ar, cigar_stride=32, buf=kernel_buffer("thread"))
    for v in (2, 3):
        buf = ExtendBuffer()
        buf.set_warp_max(0)
        buf.set_kernel_variant(v)
        out, cig = B.extend_batch_host(pr, ar, cigar_stride=32, buf=buf)
        assert (out == want[0]).all(), v
        for k in range(len(pr)):
            nops = int(out[k]["n_ops"])
            assert (cig[k, :nops] == want[1][k, :nops]).all(), (v, k)


def test_autotune_per_length_class():
    """Autotuning times every DP variant per length class, keeps the fastest,
    and later batches (per-class launches, then a captured graph) give the
    same results as the untuned path."""
    import ctypes as C
    from esperanto_gb300 import _native as N
    from esperanto_gb300.extend import ExtendBuffer, ExtendParams
    n = 30000
    ar, pr = W.synth_gotoh(21, n, 2)
    wo, wc = B.extend_batch_host(pr, ar, cigar_stride=32)
    lim = N.BatchLimitsC(300, 300 + 256, 128)
    p = ExtendParams()._c()
    buf = ExtendBuffer()
    d_arena = torch.from_numpy(ar).cuda()
    d_pairs = torch.from_numpy(pr.view(np.uint8)).cuda()
    d_out = torch.zeros(n * B.EXT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_cig = torch.zeros(n * 32, dtype=torch.int32, device="cuda")
    variants = (C.c_int * 4)()
    ms = (C.c_double * 20)()
    args = (buf.handle, B.MODE_BAND, d_pairs.data_ptr(), n, d_arena.data_ptr(), ar.nbytes, None,
            0, C.byref(lim), C.byref(p), d_out.data_ptr(), d_cig.data_ptr(), 32, None)
    buf.check(N.lib().esp_batch_autotune(*args, variants, ms))
    assert all(v in (0, 1, 2, 3) for v in variants) and all(x > 0 for x in ms)
    for it in range(4):  # per-class launches, then capture and replays
        if it:
            d_out.zero_()
            buf.check(N.lib().esp_batch_extend_device(*args))
        torch.cuda.synchronize()
        out = d_out.cpu().numpy().view(B.EXT_DTYPE)
        assert (out == wo).all()
        cig = d_cig.cpu().numpy().view(np.uint32).reshape(n, 32)
        for k in range(0, n, 101):
            assert (cig[k, :out[k]["n_ops"]] == wc[k, :out[k]["n_ops"]]).all()


def test_hint_escalation_decisions_match_oracle():
    """extend_hint's second attempt (extend.rs:392-428: a touch or a low score
    escalates to the full matrix) runs for exactly the pairs the oracle
    escalates, on the banded and the mixed-length workloads; the escalation
    rate is then the oracle's too."""
    from gpu_helpers import gpu_batch
    for shape, n in ((0, 1024), (2, 512)):
        arena, pairs = W.synth_gotoh(7, n, shape)
        cases = []
        for k in range(n):
            r, w = B.decode_pair(arena, pairs[k])
            cases.append((r, w, (int(pairs[k]["band_offset"]), 30)))
        got = gpu_batch(cases, 0, B.MODE_HINT)
        for k, (r, w, band) in enumerate(cases):
            want, esc = O.extend_hint(r, w, O.Params(), offset=band[0], with_escalation=True)
            assert got[k][0] == want.key() and got[k][2] == esc, (shape, k)


def test_large_batches_run_paired_kernel_with_same_results():
    """Band and hint batches of 2^20 pairs and more on a default handle run
    the two-pairs-per-thread kernel (2^21 band pairs: as the host pipeline's
    two chunks); the results equal the one-pair kernel's (handles forced to
    it by ESP_GOTOH_VARIANT / ESP_GOTOH_HINT_VARIANT; 2^21 pairs: four
    chunks) and, for hint batches, the oracle's on a sample."""
    import os
    from esperanto_gb300.extend import ExtendBuffer
    for mode, env, n in ((B.MODE_BAND, "ESP_GOTOH_VARIANT", 1 << 21),
                         (B.MODE_HINT, "ESP_GOTOH_HINT_VARIANT", 1 << 20)):
        arena, pairs = W.synth_gotoh(13, n, 0)
        big = B.extend_batch_host(pairs, arena, mode=mode, cigar_stride=32, buf=ExtendBuffer())
        os.environ[env] = "1"
        try:
            one = B.extend_batch_host(pairs, arena, mode=mode, cigar_stride=32,
                                      buf=ExtendBuffer())
        finally:
            del os.environ[env]
        assert (big[0] == one[0]).all()
        used = np.arange(32)[None, :] < np.minimum(big[0]["n_ops"], 32)[:, None]
        assert ((big[1] == one[1]) | ~used).all()
    rng = np.random.default_rng(1)
    for k in rng.choice(len(pairs), 200, replace=False):
        r, w = B.decode_pair(arena, pairs[k])
        want, esc = O.extend_hint(r, w, O.Params(), offset=int(pairs[k]["band_offset"]),
                                  with_escalation=True)
        o = big[0][k]
        got = (int(o["score"]), int(o["read_start"]), int(o["read_end"]), int(o["ref_start"]),
               tuple(B.cigar_of(big[1][k], int(o["n_ops"]))))
        assert got == want.key() and bool(o["escalated"]) == esc, k


def test_long_cigars_beyond_the_local_run_list():
    """CIGARs of more than 16 runs (many separated indels) leave the
    thread's local run list for their output slots; also at a capacity that
    cuts them off (ESP_ECAP, as before)."""
    rng = np.random.default_rng(41)
    cases = []
    for k in range(64):
        win = "".join(rng.choice(list("ACGT"), 400))
        read = list(win[20:380])
        for p in sorted(rng.choice(np.arange(10, 350, 12), 14 + k % 10, replace=False),
                        reverse=True):
            if rng.random() < 0.5:
                read.pop(int(p))
            else:
                read.insert(int(p), str(rng.choice(list("ACGT"))))
        cases.append(("".join(read).encode(), win.encode(), None))
    dirs = [k % 3 for k in range(len(cases))]
    assert compare(cases, dirs, kernels=("thread", "warp", "paired")) == len(cases)
    want = [O.run_dispatch(r, w, O.Params(edit_dir=d), band=None)[0].key()
            for (r, w, _), d in zip(cases, dirs)]
    assert max(len(key[4]) for key in want) > 16
    # a capacity of 20 ops: longer CIGARs report ESP_ECAP, short ones are exact
    arena, pairs, n_iv = B.pack_ascii_pairs([c[0] for c in cases], [c[1] for c in cases],
                                            [0] * len(cases), [-1] * len(cases))
    for d in range(3):
        idx = [k for k in range(len(cases)) if dirs[k] == d]
        out, cig = B.extend_batch_host(pairs[idx], arena, n_iv, E.ExtendParams(edit_dir=d),
                                       B.MODE_BAND, 20)
        for row, k in enumerate(idx):
            n_ops = len(want[k][4])
            if n_ops > 20:
                assert int(out[row]["status"]) == -3, k  # ESP_ECAP
            elif n_ops <= 18:
                o = out[row]
                assert int(o["status"]) == 0, k
                got = (int(o["score"]), int(o["read_start"]), int(o["read_end"]),
                       int(o["ref_start"]), tuple(B.cigar_of(cig[row], int(o["n_ops"]))))
                assert got == want[k], k


def test_cigar_capacity_exact_fit():
    """A CIGAR of up to 16 runs needs exactly its final length in capacity:
    a stride equal to the oracle's op count succeeds bit-exactly, one less
    reports ESP_ECAP."""
    rng = np.random.default_rng(43)
    for k in range(24):
        win = "".join(rng.choice(list("ACGT"), 260))
        read = list(win[30:230])
        for p in sorted(rng.choice(np.arange(20, 180, 15), 1 + k % 6, replace=False),
                        reverse=True):
            if rng.random() < 0.5:
                read.pop(int(p))
            else:
                read.insert(int(p), str(rng.choice(list("ACGT"))))
        read = ("".join(rng.choice(list("ACGT"), 1 + k % 4)) + "".join(read)).encode()
        want = O.run_dispatch(read, win.encode(), O.Params(), band=None)[0].key()
        n_ops = len(want[4])
        arena, pairs, n_iv = B.pack_ascii_pairs([read], [win.encode()], [0], [-1])
        for kern in ("warp", "thread"):
            buf = kernel_buffer(kern)
            out, cig = B.extend_batch_host(pairs, arena, n_iv, E.ExtendParams(), B.MODE_BAND,
                                           n_ops, buf=buf)
            o = out[0]
            assert int(o["status"]) == 0, (k, n_ops, kern)
            got = (int(o["score"]), int(o["read_start"]), int(o["read_end"]),
                   int(o["ref_start"]), tuple(B.cigar_of(cig[0], int(o["n_ops"]))))
            assert got == want, (k, kern)
            if n_ops > 1:
                out, _ = B.extend_batch_host(pairs, arena, n_iv, E.ExtendParams(), B.MODE_BAND,
                                             n_ops - 1, buf=buf)
                assert int(out[0]["status"]) == -3, (k, kern)  # ESP_ECAP
