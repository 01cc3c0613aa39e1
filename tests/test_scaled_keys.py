"""Host model of the DP kernels' cell formulation (gotoh.cu dp_column /
dp_column2): every H, E and F is held as a scaled key 4v + tag, so that one
integer max per quantity performs the reference's selection and tie order
(extend.rs:737-793, as the oracle's extend.c restates it):

* E = e_up + ext unless h_up + open_ext is at least as large (open on ties);
  F likewise from the left; key tag 1 = E opened here, 2 = F opened here;
* H starts at 0 (START), then takes F, E, diag in that order whenever the
  candidate is >= the current value; H == 0 is START again.  With the E key
  lifted by 1, the diagonal floored at key 3 and F's key as is, one 3-way
  max of (diag, E + 1, F) yields the same value and direction: diag (tag 2)
  beats E (1) beats F (0) on ties, and any value <= 0 loses to START (key 3,
  value 0).

The model draws cells over the score domain the kernels accept (H up to
8191, substitution scores in [-32, 31], 4 (open + ext) <= 8000) with
out-of-window E / F inputs as the kernels' sentinel, and compares value,
direction and both opened flags with the reference's cascade.
"""
import random

NEG = None          # the reference's out-of-window E / F
NEG4 = -32768       # the kernels' scaled sentinel for it
H_DIAG, H_FROM_E, H_FROM_F, H_START = 0, 1, 2, 3


def reference_cell(h_up, e_up, h_left, f_left, h_diag, s, open_ext, ext):
    e_open = h_up + open_ext
    e_ext = None if e_up is NEG else e_up + ext
    if e_ext is not None and e_ext > e_open:
        e, e_opened = e_ext, False
    else:
        e, e_opened = e_open, True
    f_open = h_left + open_ext
    f_ext = None if f_left is NEG else f_left + ext
    if f_ext is not None and f_ext > f_open:
        f, f_opened = f_ext, False
    else:
        f, f_opened = f_open, True
    diag = h_diag + s
    h, hdir = 0, H_START
    if not h > f:
        h, hdir = f, H_FROM_F
    if not h > e:
        h, hdir = e, H_FROM_E
    if not h > diag:
        h, hdir = diag, H_DIAG
    if h == 0:
        hdir = H_START
    return h, hdir, e, e_opened, f, f_opened


def kernel_cell(h_up, e_up, h_left, f_left, h_diag, s, open_ext, ext):
    ex4, oe1, oe4 = 4 * ext, 4 * open_ext - 1, 4 * open_ext
    up_h, left, d = 4 * h_up + 2, 4 * h_left + 2, 4 * h_diag + 2
    up_e = NEG4 if e_up is NEG else 4 * e_up
    fl = NEG4 if f_left is NEG else 4 * f_left
    kE = max(up_e + ex4, up_h + oe1)
    kF = max(fl + ex4, left + oe4)
    E4, F4 = kE & ~3, kF & ~3
    kd = max(d + 4 * s, 3)
    key = max(kd, E4 + 1, F4)
    Hp = (key & ~3) | 2
    tag = key & 3
    flags = (kE | kF) & 3
    hdir = {2: H_DIAG, 1: H_FROM_E, 0: H_FROM_F, 3: H_START}[tag]
    return (Hp - 2) // 4, hdir, E4 // 4, bool(flags & 1), F4 // 4, bool(flags & 2)


def test_scaled_keys_equal_the_reference_cascade():
    rng = random.Random(3)
    params = [(-6, -2), (-800, -400), (-3, -1), (-2000, 0), (-1, 0)]
    for k in range(200000):
        open_ext, ext = params[k % len(params)]
        hv = lambda: rng.choice([0, 0, 1, 2, rng.randrange(0, 60), rng.randrange(0, 8192)])
        ef = lambda: NEG if rng.random() < 0.15 else rng.choice(
            [rng.randrange(open_ext - 10, 60), hv() + open_ext])
        cell = (hv(), ef(), hv(), ef(), hv(), rng.randrange(-32, 32), open_ext, ext)
        want = reference_cell(*cell)
        got = kernel_cell(*cell)
        if want[0] < 0:  # H is never negative: START floors it
            raise AssertionError(cell)
        assert got == want, (cell, got, want)
