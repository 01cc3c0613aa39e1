"""Input generators restated from the reference's own unit tests.

These reproduce, byte for byte, the sequences the reference tests feed to the
hot path, so that its known answers and seeded sweeps can be replayed here:

* ``body(n)``      crates/map/src/fragment.rs:141-151 (xorshift seed 0xe911da37)
* ``revcomp``      crates/map/src/align.rs:2518-2532 (N stays N)
* ``Rng``          crates/map/src/extend.rs:2481-2500 (xorshift 13/7/17 over ACGTN)
* ``rand_seq``     crates/map/src/extend.rs:2502-2505
* ``rand_window``  crates/map/src/extend.rs:2507-2525
"""
from __future__ import annotations

MASK64 = (1 << 64) - 1


def body(n: int) -> bytes:
    state = 0xE911DA37
    out = bytearray()
    for _ in range(n):
        state ^= (state << 13) & MASK64
        state ^= state >> 7
        state ^= (state << 17) & MASK64
        out.append(b"ACGT"[state & 3])
    return bytes(out)


_COMP = {ord("A"): ord("T"), ord("C"): ord("G"), ord("G"): ord("C"), ord("T"): ord("A"),
         ord("a"): ord("T"), ord("c"): ord("G"), ord("g"): ord("C"), ord("t"): ord("A")}


def revcomp(seq: bytes) -> bytes:
    return bytes(_COMP.get(b, ord("N")) for b in reversed(seq))


class Rng:
    def __init__(self, seed: int):
        self.s = seed & MASK64

    def next(self) -> int:
        x = self.s
        x ^= (x << 13) & MASK64
        x ^= x >> 7
        x ^= (x << 17) & MASK64
        self.s = x
        return x

    def below(self, n: int) -> int:
        return self.next() % n

    def base(self) -> int:
        return b"ACGTN"[self.below(5)]


def rand_seq(rng: Rng, n: int) -> bytes:
    return bytes(rng.base() for _ in range(n))


def rand_window(rng: Rng, read: bytes, n: int) -> bytes:
    w = bytearray(rand_seq(rng, n))
    if n > len(read):
        off = rng.below(n - len(read) + 1)
        k = 0
        while k < len(read) and off + k < n:
            b = read[k]
            w[off + k] = rng.base() if rng.below(8) == 0 else b
            if rng.below(16) == 0:
                k += 2
            else:
                k += 1
    return bytes(w)


DIRS = (0, 1, 2)  # EditDir Off, Ag, Tc


def sweep_full_matrix():
    """Cases of avx2_full_matrix_matches_scalar (extend.rs:2578-2627):
    yields (read, window, edit_dir, ctx)."""
    rng = Rng(0x9E3779B97F4A7C15)
    lens_m = [1, 2, 3, 7, 8, 15, 16, 17, 31, 32, 33, 63, 64, 100, 150, 151, 200]
    lens_n = [1, 2, 3, 7, 8, 15, 16, 17, 31, 48, 63, 64, 100, 127, 255, 257, 1000, 3000]
    for m in lens_m:
        for n in lens_n:
            for rep in range(3):
                read = rand_seq(rng, m)
                win = rand_seq(rng, n) if (rep == 2 or n < m) else rand_window(rng, read, n)
                d = DIRS[rng.below(3)]
                yield read, win, d, f"m={m} n={n} rep={rep}"
    for rep in range(3):
        read = rand_seq(rng, 150)
        win = rand_seq(rng, 20000) if rep == 2 else rand_window(rng, read, 20000)
        yield read, win, 1, f"long rep={rep}"


def sweep_full_block_boundaries():
    """avx2_full_matrix_block_boundaries (extend.rs:2632-2659)."""
    rng = Rng(0x0F1E2D3C4B5A6978)
    for m in range(14, 21):
        for n in range(1, 21):
            for rep in range(4):
                read = rand_seq(rng, m)
                if rep & 1 == 0 and n >= m:
                    win = rand_window(rng, read, n)
                else:
                    win = rand_seq(rng, n)
                yield read, win, DIRS[rep % 3], f"m={m} n={n} rep={rep}"
    for n in [30, 31, 32, 33, 47, 63, 64, 65]:
        read = rand_seq(rng, 17)
        win = rand_window(rng, read, n)
        yield read, win, 2, f"tail n={n}"


def sweep_band():
    """avx2_band_matches_scalar (extend.rs:2723-2822): yields
    (read, window, edit_dir, offset, half, ctx)."""
    rng = Rng(0xA5A55A5AC3C33C3C)
    shapes = [(8, 9), (8, 40), (15, 16), (16, 16), (17, 33), (20, 200), (31, 31), (32, 64),
              (60, 61), (60, 300), (100, 300), (150, 151), (150, 1000), (40, 20), (17, 9)]
    for m, n in shapes:
        mn = max(m, n)
        halfs = [0, 1, 2, 30, mn + 5] if n <= 64 else [0, 1, 2, 30, 300]
        for rep in range(2):
            read = rand_seq(rng, m)
            win = rand_seq(rng, n) if rep == 1 else rand_window(rng, read, n)
            for half in halfs:
                hh = min(half, mn)
                for offset in [-hh - 5, -1, 0, 5, n - m, n, n + hh + 5, 4 * n]:
                    d = DIRS[rng.below(3)]
                    yield read, win, d, offset, half, f"m={m} n={n} rep={rep} h={half} o={offset}"
    for rep in range(3):
        read = rand_seq(rng, 150)
        win = rand_seq(rng, 20000) if rep == 2 else rand_window(rng, read, 20000)
        for offset, half in [(-40, 30), (0, 30), (5000, 30), (19850, 30), (-20000, 20000),
                             (20000, 20000)]:
            yield read, win, 1, offset, half, f"long rep={rep} o={offset} h={half}"


def sweep_band_block_boundaries():
    """avx2_band_block_boundaries (extend.rs:2828-2863)."""
    rng = Rng(0x13579BDF2468ACE0)
    halfs = [0, 1, 2, 7, 8, 15, 16, 17, 30, 31, 32, 33, 48]
    for m in range(8, 25):
        for dn in [0, 1, 15, 16, 17, 31, 32, 33]:
            n = m + dn
            for rep in range(2):
                read = rand_seq(rng, m)
                win = rand_seq(rng, n) if rep == 1 else rand_window(rng, read, n)
                for half in halfs:
                    offset = rng.below(120) - 60 + (n - m)
                    yield read, win, DIRS[rep % 3], offset, half, f"blk m={m} n={n} h={half} o={offset}"
