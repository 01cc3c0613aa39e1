"""The pipeline batching hook (crates/map/src/pipeline.rs:394-403): a chunk
collector filled from several host threads returns, for every request and
in input order, exactly what the per-call entry point returns -- and what
the oracle returns -- over a chunk of extend_hint, run_band, extend and
EA-Myers requests of every kind, including the entry points' guards (empty
reads, Myers lengths beyond the single block and beyond 256), N and
lowercase bases; a second round after reset does the same."""
import random
import threading

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import oracle as O  # noqa: E402
import esperanto_gb300 as E  # noqa: E402
from esperanto_gb300 import EspError  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300 import engine_myers, myers_ea  # noqa: E402
from esperanto_gb300.chunk import Chunk  # noqa: E402
import workloads as W  # noqa: E402


def _requests(seed, n_reads):
    """(kind, args) requests of one chunk: the 150 x 214 workload's pairs
    through extend_hint (and a tenth through run_band / extend), each read's
    Myers filters, and edge cases."""
    rng = random.Random(seed)
    arena, pairs = W.synth_gotoh(seed, n_reads, 0)
    reqs = []
    for k in range(n_reads):
        r, w = B.decode_pair(arena, pairs[k])
        if k % 37 == 5:  # N runs and lowercase (base_code folding)
            r = r[:40] + b"NN" + r[42:100].lower() + r[100:]
        reqs.append(("hint", r, w, 32))
        if k % 10 == 3:
            reqs.append(("band", r, w, (32, 32)))
        if k % 10 == 7:
            reqs.append(("extend", r, w[20:200]))
        kind = ("myers_ea::long::infix_best_start", "myers_ea::long::infix_best_end",
                "myers_ea::long::infix", "engine::myers::infix",
                "engine::myers::global")[k % 5]
        reqs.append(("myers", kind, r, w))
        if k % 9 == 0:
            reqs.append(("myers", "myers_ea::infix_best_end", r[:100], w))
            reqs.append(("myers", "myers_ea::infix_best_start", r[20:120], w))
            reqs.append(("myers", "myers_ea::infix", r[:64], w))
    # guards: empty read / window, Myers m = 0 and m > 256
    long_read = bytes(rng.choice(b"ACGT") for _ in range(300))
    reqs += [("hint", b"", b"ACGTACGT", 0), ("hint", b"ACGTACGT", b"", 0),
             ("band", b"ACGT", b"ACGTT", None),
             ("myers", "myers_ea::long::infix_best_end", b"", b"ACGT"),
             ("myers", "myers_ea::long::infix_best_start", long_read, long_read + b"A"),
             ("myers", "myers_ea::infix", long_read, long_read)]
    return reqs


def _add(ch, q):
    if q[0] == "hint":
        return ch.add_extend_hint(q[1], q[2], E.DiagHint(q[3]))
    if q[0] == "band":
        return ch.add_run_band(q[1], q[2], q[3])
    if q[0] == "extend":
        return ch.add_extend(q[1], q[2])
    return ch.add_myers(q[1], q[2], q[3])


def _per_call(q):
    if q[0] == "hint":
        return E.extend_hint(q[1], q[2], hint=E.DiagHint(q[3])).key()
    if q[0] == "band":
        return E.run_band(q[1], q[2], band=q[3])[0].key()
    if q[0] == "extend":
        return E.extend(q[1], q[2]).key()
    kind, r, t = q[1], q[2], q[3]
    if kind == "engine::myers::infix":
        return (engine_myers.infix(r, t), 0)
    if kind == "engine::myers::global":
        return (engine_myers.global_(r, t), 0)
    ns = myers_ea.long if kind.startswith("myers_ea::long::") else myers_ea
    fn = kind.rsplit("::", 1)[1]
    res = getattr(ns, fn)(r, t)
    return res if isinstance(res, tuple) else (res, 0)


def _oracle(q):
    if q[0] == "hint":
        return O.extend_hint(q[1], q[2], offset=q[3]).key()
    if q[0] == "band":
        return O.run_dispatch(q[1], q[2], band=q[3])[0].key()
    if q[0] == "extend":
        return O.extend(q[1], q[2]).key()
    kind, r, t = q[1], q[2], q[3]
    if kind == "engine::myers::infix":
        return (O.engine_infix(r, t), 0)
    if kind == "engine::myers::global":
        return (O.engine_global(r, t), 0)
    fn = {"myers_ea::infix": lambda: (O.myers_infix(r, t), 0),
          "myers_ea::infix_best_end": lambda: O.myers_infix_best_end(r, t),
          "myers_ea::infix_best_start": lambda: O.myers_infix_best_start(r, t),
          "myers_ea::long::infix": lambda: (O.myers_long_infix(r, t), 0),
          "myers_ea::long::infix_best_end": lambda: O.myers_long_infix_best_end(r, t),
          "myers_ea::long::infix_best_start": lambda: O.myers_long_infix_best_start(r, t)}
    return tuple(fn[kind]())


def test_chunk_collector_equals_per_call_and_oracle():
    ch = Chunk(cigar_stride=64)
    for rnd, seed in enumerate((41, 42)):
        reqs = _requests(seed, 3000)
        # four worker threads add interleaved slices, as rayon workers would
        idx = [None] * len(reqs)

        def worker(t):
            for k in range(t, len(reqs), 4):
                idx[k] = _add(ch, reqs[k])
        ths = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        assert sorted(idx) == list(range(len(reqs))) and len(ch) == len(reqs)
        ch.run()
        with pytest.raises(EspError):  # a run chunk takes no more requests until reset
            ch.add_extend(b"ACGT", b"ACGT")
        for k, q in enumerate(reqs):
            got = ch.extension(idx[k]).key() if q[0] != "myers" else ch.myers(idx[k])
            assert got == _per_call(q), (rnd, k, q[0], q[1] if q[0] == "myers" else "")
            if k % 3 == 0 or q[0] == "myers":
                assert got == _oracle(q), (rnd, k)
        ch.reset()
        assert len(ch) == 0
    ch.close()


def test_chunk_guards_match_the_entry_points():
    ch = Chunk(cigar_stride=8)
    read = b"ACGT" * 40  # 160 bases: above the single-block Myers limit
    with pytest.raises(EspError):
        ch.add_myers("myers_ea::infix_best_end", read, read)
    with pytest.raises(EspError):
        ch.add_myers("engine::myers::global", b"", read)
    # a CIGAR longer than the chunk's stride reports ESP_ECAP, as the
    # per-call drop-in with that capacity does
    win = b"ACGTTGCA" * 30
    r = bytearray(win[10:230])
    for p in (200, 170, 140, 110, 80, 50, 20):
        del r[p]
    i = ch.add_extend(bytes(r), win)
    ch.run()
    want = O.extend(bytes(r), win)
    if len(want.cigar) > 8:
        with pytest.raises(EspError) as ei:
            ch.extension(i)
        assert ei.value.code == -3
    else:
        assert ch.extension(i).key() == want.key()
    ch.close()
