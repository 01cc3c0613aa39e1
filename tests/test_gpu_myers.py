"""GPU parity for the EA-Myers filters (myers_ea.rs, engine/src/myers.rs)
against the oracle, which is itself pinned to a brute-force edit-distance DP
(tests/test_oracle_sweeps.py)."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import oracle as O  # noqa: E402
from esperanto_gb300 import EspError  # noqa: E402
from esperanto_gb300 import batch as B  # noqa: E402
from esperanto_gb300 import engine_myers, myers_ea  # noqa: E402
import workloads as W  # noqa: E402


def _case(rng, m, n, alpha="ACGT"):
    text = bytes(rng.choice(alpha.encode()) for _ in range(n))
    if n >= m and rng.random() < 0.6:
        s = rng.randrange(0, n - m + 1)
        read = bytearray(text[s:s + m].upper().replace(b"N", b"C"))
        for _ in range(rng.randrange(0, 7)):
            read[rng.randrange(m)] = rng.choice(b"ACGTN")
        read = bytes(read)
    else:
        read = bytes(rng.choice(b"ACGTN") for _ in range(m))
    return read, text


MS = [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 150, 200, 255, 256]


@pytest.mark.parametrize("m", MS)
def test_per_call_entry_points(m):
    rng = random.Random(77 + m)
    for rep in range(6):
        n = rng.choice([0, 1, m, m + 50, 2 * m + 3, 400])
        read, text = _case(rng, m, n, "ACGTacgtN" if rep % 2 else "ACGT")
        assert myers_ea.long.infix_best_end(read, text) == O.myers_long_infix_best_end(read, text)
        assert myers_ea.long.infix_best_start(read, text) == O.myers_long_infix_best_start(read, text)
        assert myers_ea.long.infix(read, text) == O.myers_long_infix(read, text)
        if m <= 128:
            assert myers_ea.infix_best_end(read, text) == O.myers_infix_best_end(read, text)
            assert myers_ea.infix_best_start(read, text) == O.myers_infix_best_start(read, text)
            assert myers_ea.infix(read, text) == O.myers_infix(read, text)
        else:
            with pytest.raises(EspError):
                myers_ea.infix_best_end(read, text)
        assert engine_myers.infix(read, text) == O.engine_infix(read, text)
        assert engine_myers.global_(read, text) == O.engine_global(read, text)


def test_guards():
    assert myers_ea.infix_best_end(b"", b"ACGT") == (0, 0)
    assert myers_ea.infix_best_start(b"", b"ACGT") == (0, 0)
    assert myers_ea.long.infix_best_end(b"A" * 300, b"ACGT") == (300, 0)
    assert myers_ea.long.infix_best_start(b"A" * 300, b"ACGT") == (300, 0)
    with pytest.raises(EspError):
        engine_myers.infix(b"", b"ACGT")
    with pytest.raises(EspError):
        engine_myers.global_(b"A" * 257, b"ACGT")


def _oracle_batch(arena, pairs, n_iv, mode):
    out = []
    for k in range(len(pairs)):
        p = {"read_pos": pairs[k]["read_pos"], "read_len": pairs[k]["read_len"],
             "win_pos": pairs[k]["text_pos"], "win_len": pairs[k]["text_len"],
             "n_first": pairs[k]["n_first"], "n_read": pairs[k]["n_read"],
             "n_win": pairs[k]["n_text"]}
        r, t = B.decode_pair(arena, p, n_iv)
        if mode == B.MYERS_BEST_END:
            out.append(O.myers_long_infix_best_end(r, t))
        elif mode == B.MYERS_BEST_START:
            out.append(O.myers_long_infix_best_start(r, t))
        else:
            out.append((O.engine_global(r, t), 0))
    return out


@pytest.mark.parametrize("mode", [B.MYERS_BEST_END, B.MYERS_BEST_START, B.MYERS_GLOBAL])
def test_batch_mixed_lengths_with_n(mode):
    rng = random.Random(9 + mode)
    reads, texts = [], []
    for k in range(1500):
        m = rng.choice(MS)
        n = rng.randrange(0, 400)
        r, t = _case(rng, m, n, "ACGTN" if k % 5 == 0 else "ACGT")
        reads.append(r)
        texts.append(t)
    arena, pairs, n_iv = B.pack_ascii_myers(reads, texts)
    got = B.myers_batch_host(pairs, arena, n_iv, mode)
    assert (got["status"] == 0).all()
    want = _oracle_batch(arena, pairs, n_iv, mode)
    for k, (d, p) in enumerate(want):
        assert (int(got[k]["dist"]), int(got[k]["pos"])) == (d, p), k


def test_myers_150x200_subset():
    arena, pairs = W.synth_myers(2, 20000)
    got = B.myers_batch_host(pairs, arena)
    want = _oracle_batch(arena, pairs, None, B.MYERS_BEST_END)
    assert [(int(g["dist"]), int(g["pos"])) for g in got] == want


def test_host_batch_pipeline_chunks():
    """Host batches of 2^18 pairs and more run as eight chunks whose copies
    overlap the neighbouring chunks' kernels: the results equal those of
    unchunked calls on the same pairs, also when the pairs reference the
    arena out of order (each chunk then needs most of the arena), and the
    oracle on a sample."""
    arena, pairs = W.synth_myers(5, 300000)
    rng = np.random.default_rng(3)
    for order in (np.arange(len(pairs)), rng.permutation(len(pairs))):
        p = pairs[order]
        got = B.myers_batch_host(p, arena)
        half = len(p) // 2  # below the chunking size: one launch each
        want = np.concatenate([B.myers_batch_host(p[:half], arena),
                               B.myers_batch_host(p[half:], arena)])
        assert (got == want).all()
    sample = [int(k) for k in rng.choice(len(pairs), 300, replace=False)]
    got = B.myers_batch_host(pairs, arena)
    want = _oracle_batch(arena, pairs[sample], None, B.MYERS_BEST_END)
    assert [(int(got[k]["dist"]), int(got[k]["pos"])) for k in sample] == want
