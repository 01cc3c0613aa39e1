// gotoh.cu -- GB300 banded / full-matrix affine-gap (Gotoh) local alignment
// with traceback to CIGAR, bit-exact with the reference's scalar kernel
// (crates/map/src/extend.rs:606-1068).
//
// Execution model: one thread owns one read x window pair (inter-sequence
// parallelism).  A warp takes 32 consecutive entries of a length-sorted work
// list from a device queue (persistent kernel), so the lanes of a warp run the
// same loop trip counts and their scratch accesses coalesce.
//
// DP layout: the matrix is swept in strips of 8 rows.  Inside a strip the
// thread walks the strip's column range left to right and evaluates the 8
// cells of each column top to bottom, all in registers:
//   * H/F of column j-1 for each of the 8 rows ride in registers (left deps),
//   * H/E of the row above the strip come from a per-thread row buffer (one
//     packed int16x2 word per column) that the strip's last row rewrites in
//     place, so row-buffer traffic is 8 bytes per column per 8 cells,
//   * the 4 traceback bits of the 8 cells are packed into one 32-bit word
//     per (strip, column): 2 bits H source per row in the low half-word and
//     (E opened, F opened) per row in the high half-word.
//
// Scaled-key arithmetic (what makes the reference's tie cascade cheap):
// every score is held as 4*v plus a 2-bit tag so that a plain integer max
// performs both the value comparison and the reference's tie preference.
//   H is held as Hp = 4H + 2.
//   E key: max(Hp_up + 4*open_ext - 1, E4_up + 4*ext): low bit 1 <=> opened,
//          and an open/extend tie resolves to "open" as `better` (strict >)
//          does at extend.rs:731.
//   F key: max(Hp_left + 4*open_ext, F4_left + 4*ext): bit 1 <=> opened.
//   H key: max(4*diag + 2, 4E + 1, 4F + 0, 3): among equal values diag
//          beats E beats F (the cascade order of extend.rs:764-777), and the
//          START tag 3 wins whenever the maximum is 0 (the zero-floor rewrite
//          of extend.rs:780-782).  hsrc = key & 3: 3 start, 2 diag, 1 E, 0 F.
// Out-of-window cells present H = 0, E = F = NEG to their neighbours exactly
// as the scalar kernel's margins do (extend.rs:718-759).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <type_traits>

#include "esp_device.cuh"
#include "esp_internal.h"

namespace esp {

static constexpr int NEG4 = -32768;  // E/F sentinel in scaled units (int16 min)
static constexpr int STRIP = 8;

struct Geo {
    int off, half, n;
    __device__ __forceinline__ int c(int i) const {
        int x = off + i;
        return x < 1 ? 1 : (x > n ? n : x);
    }
    __device__ __forceinline__ int lo(int i) const {
        int v = c(i) - half;
        return v > 1 ? v : 1;
    }
    __device__ __forceinline__ int hi(int i) const {
        int v = c(i) + half;
        return v < n ? v : n;
    }
};

struct Seq {
    const uint8_t *arena;
    uint64_t pos;
    const esp_n_interval *iv;
    uint32_t cnt;
    __device__ __forceinline__ uint32_t code(int64_t q) const {
        return code5(arena, pos, iv, cnt, q);
    }
};

// Row-max keys are Hp * 32768 + (32767 - j): 32 bits while Hp < 65536 (the
// int16 domain); the wide kernel keeps them in 64 bits.
template <bool WIDE>
struct StripT {
    using RK = typename std::conditional<WIDE, long long, int>::type;
    int Hl[STRIP], Fl[STRIP];
    RK rk[STRIP];
    uint32_t l0[STRIP], l1[STRIP];
    int lo[STRIP], hi[STRIP];
};
using Strip = StripT<false>;

__device__ __forceinline__ uint32_t mad_u32(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;  // integer multiply-add: issues on the FMA pipe, off the saturated ALU pipe
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// a & m and (a & m) | o as opaque logic ops, so that the compiler keeps the
// differences below as adds instead of folding them back into logic.
__device__ __forceinline__ uint32_t and_u32(uint32_t a, uint32_t m) {
    uint32_t d;
    asm("and.b32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(m));
    return d;
}

// (a | b) & m in one LOP3
__device__ __forceinline__ uint32_t or_and_u32(uint32_t a, uint32_t b, uint32_t m) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0xA8;" : "=r"(d) : "r"(a), "r"(b), "r"(m));
    return d;
}

__device__ __forceinline__ uint32_t and_or_u32(uint32_t a, uint32_t m, uint32_t o) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0xEA;" : "=r"(d) : "r"(a), "r"(m), "r"(o));
    return d;
}

// One column of one strip.  upH/upE enter as the row above the strip at
// column j and leave as the strip's last row at column j; `diag` is the row
// above at column j-1; cj = 32767 - j (row-max key tie order).  MASK = 1
// tests every cell against its row window (strip ramps); MASK = 0 is the
// strip interior where all 8 cells are in window.
template <int MASK, bool WIDE = false>
__device__ __forceinline__ uint32_t dp_column(StripT<WIDE> &S, const GotohConst &K, int j,
                                              uint32_t sel, uint32_t cj, int &upH, int &upE,
                                              int diag) {
    uint32_t wa = 0, wb = 0;
    int d = diag;
#pragma unroll
    for (int r = 0; r < STRIP; r++) {
        int left = S.Hl[r];
        int kE = max(upE + K.ex4, upH + K.oe1);
        int kF = max(S.Fl[r] + K.ex4, left + K.oe4);
        // kE = 0 or 1 and kF = 0 or 2 (mod 4): the two opened flags are
        // (kE | kF) & 3 (one LOP3); the E tag is E4 + 1 and the key's tag
        // key - Hp + 2 -- adds, which also issue on the FMA pipe, instead of
        // logic ops on the saturated ALU pipe
        int E4 = (int)and_u32((uint32_t)kE, ~3u);
        int F4 = (int)and_u32((uint32_t)kF, ~3u);
        int kd = max(d + prmt_sx(S.l0[r], S.l1[r], sel), 3);  // START tag 3 folded in
        int key = max(max(kd, E4 + 1), F4);
        int Hp = (int)and_or_u32((uint32_t)key, ~3u, 2u);
        wa = mad_u32(wa, 4u, (uint32_t)(key - Hp + 2));
        wb = mad_u32(wb, 4u, or_and_u32((uint32_t)kE, (uint32_t)kF, 3u));
        typename StripT<WIDE>::RK rkey;
        if constexpr (WIDE)
            rkey = ((long long)Hp << 15) | (long long)cj;
        else
            rkey = (int)mad_u32((uint32_t)Hp, 32768u, cj);
        if (MASK) {
            // An out-of-window cell shows H = 0, E = NEG to the row below and
            // leaves its row's state alone: before the window that is still
            // the start state, after it Hl keeps H at the window's last
            // column (the strip's bookkeeping reads it; the cells of the row
            // below that follow are out of their window too, as hi(i+1) <=
            // hi(i) + 1).
            const bool in = (j >= S.lo[r]) & (j <= S.hi[r]);
            if (in) {
                S.rk[r] = max(S.rk[r], rkey);
                S.Hl[r] = Hp;
                S.Fl[r] = F4;
            }
            upH = in ? Hp : 2;
            upE = in ? E4 : NEG4;
        } else {
            S.rk[r] = max(S.rk[r], rkey);
            S.Hl[r] = Hp;
            S.Fl[r] = F4;
            upH = Hp;
            upE = E4;
        }
        d = left;
    }
    return __byte_perm(wa, wb, 0x5410);
}

struct FillResult {
    int bestHp, best_i, best_j;
    int trow;
    bool tleft, tclamp;
};

// Columns [a, b] of the current strip.  Window codes are fetched 16 at a
// time.  CHECK = true (strip ramps) tests the row-buffer read (the row above
// has a value only up to phi) and write (the strip's last row starts at
// lo7) per column; the interior needs neither test.
template <int MASK, bool CHECK, bool HASN>
__device__ __forceinline__ void dp_cols(Strip &S, const GotohConst &K, int a, int b, int &diag,
                                        const Seq &win, uint32_t *rb, int plo, int phi, int lo7,
                                        uint32_t *tbp) {
    uint32_t *rbr = rb + (size_t)(a - plo) * 32;
    uint32_t cj = 32767u - (uint32_t)a;
    // Interior: the row above is read two columns ahead of its use (the
    // L2 round trip of a row-buffer line is longer than one column of
    // arithmetic).  A slot is rewritten only at or after the column that
    // reads it, so the values fetched early are still the row above.
    uint32_t wn0 = 0, wn1 = 0;
    if (!CHECK) {
        wn0 = rbr[0];
        if (a + 1 <= b) wn1 = rbr[32];
    }
    for (int j = a; j <= b;) {
        uint32_t cw = load16(win.arena, win.pos + (uint64_t)(j - 1));
        uint32_t nm = HASN ? nmask16(win.iv, win.cnt, j - 1) : 0u;
        int cnt = min(16, b - j + 1);
#pragma unroll 1  // measured: the rolled loop beats unroll 2 (+13%) and 4
        for (int k = 0; k < cnt; k++, j++) {
            uint32_t code = HASN ? ((cw >> 30) | ((nm >> 29) & 4u)) : (cw >> 30);
            cw <<= 2;
            if (HASN) nm <<= 1;
            uint32_t sel = code * 0x1111u + 0x8880u;
            int bH = 2, bE = NEG4;
            if (!CHECK || j <= phi) {
                uint32_t w;
                if (CHECK) {
                    w = *rbr;
                } else {
                    w = wn0;
                    wn0 = wn1;
                    if (j + 2 <= b) wn1 = rbr[64];
                }
                bH = (int)(w & 0xffffu);
                bE = ((int)w) >> 16;
            }
            int upH = bH, upE = bE;
            uint32_t word = dp_column<MASK>(S, K, j, sel, cj, upH, upE, diag);
            diag = bH;
            uint32_t packed = __byte_perm((uint32_t)upH, (uint32_t)upE, 0x5410);
            if (CHECK) {
                if (j >= lo7) rb[(size_t)(j - lo7) * 32] = packed;
            } else {
                rbr[(ptrdiff_t)(plo - lo7) * 32] = packed;  // row-buffer slot j - lo7
            }
            *tbp = word;
            tbp += 32;
            rbr += 32;
            cj--;
        }
    }
}

// Fill the DP for one pair; traceback words land in tb (stride sw per strip).
// The row buffer holds sw words: strip 0 reads row 0 (H = 0, E = NEG on every
// column, extend.rs:664-681) from a prefilled copy, later strips read the last
// row of the previous strip, which each strip rewrites in place (a slot is
// always read at or before the column that overwrites it, since the strip's
// window start lo7 never precedes the previous row's start plo).
template <bool HASN>
__device__ FillResult dp_fill(const GotohConst &K, const uint32_t *__restrict__ s_lut, int m,
                              int n, const Geo &g, const Seq &read, const Seq &win,
                              uint32_t *tb, int sw, uint32_t *rb) {
    FillResult R;
    R.bestHp = 2;
    R.best_i = 0;
    R.best_j = 0;
    R.trow = 0;
    R.tleft = false;
    R.tclamp = false;
    int nstrips = (m + STRIP - 1) / STRIP;
    int plo = g.lo(1), phi = g.hi(min(STRIP, m));
    {
        const uint32_t row0 = __byte_perm(2u, (uint32_t)NEG4, 0x5410);
        for (int k = 0; k <= phi - plo; k++) rb[(size_t)k * 32] = row0;
    }
    Strip S;
    for (int s = 0; s < nstrips; s++) {
        int i0 = s * STRIP + 1;
        int nact = min(STRIP, m - i0 + 1);
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            S.lo[r] = g.lo(i0 + r);
            S.hi[r] = g.hi(i0 + r);
            S.Hl[r] = 2;
            S.Fl[r] = NEG4;
            S.rk[r] = -1;
        }
        int clo = S.lo[0];
        int chi = g.hi(i0 + nact - 1);
        int lo7 = S.lo[STRIP - 1];
        int hi0 = S.hi[0];
        // read codes of the strip's rows -> per-row substitution words
        uint32_t rw = load16(read.arena, read.pos + (uint64_t)(i0 - 1));
        uint32_t rn = read.cnt ? nmask16(read.iv, read.cnt, i0 - 1) : 0u;
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            uint32_t c = (rw >> (30 - 2 * r)) & 3u;
            if ((rn >> (31 - r)) & 1u) c = 4;
            S.l0[r] = s_lut[2 * c];
            S.l1[r] = s_lut[2 * c + 1];
        }
        int diag = 2;
        if (clo - 1 >= plo && clo - 1 <= phi)
            diag = (int)(rb[(size_t)(clo - 1 - plo) * 32] & 0xffffu);
        uint32_t *tbp = tb + (size_t)s * sw * 32;
        int a_end = min(lo7, chi);
        dp_cols<1, true, HASN>(S, K, clo, a_end, diag, win, rb, plo, phi, lo7, tbp);
        int b_beg = lo7 + 1, b_end = min(hi0 - 1, chi);
        if (b_beg <= b_end)
            dp_cols<0, false, HASN>(S, K, b_beg, b_end, diag, win, rb, plo, phi, lo7,
                                    tbp + (size_t)(b_beg - clo) * 32);
        int c_beg = max(lo7 + 1, hi0);
        // the row windows again rather than kept live across the interior
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            S.lo[r] = g.lo(i0 + r);
            S.hi[r] = g.hi(i0 + r);
        }
        if (c_beg <= chi)
            dp_cols<1, true, HASN>(S, K, c_beg, chi, diag, win, rb, plo, phi, lo7,
                                   tbp + (size_t)(c_beg - clo) * 32);
        // row bookkeeping in row order (extend.rs:795-827)
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            if (r < nact) {
                int rowHp = S.rk[r] >> 15;
                int argj = 32767 - (S.rk[r] & 32767);
                if (R.trow == 0) {
                    if (argj == S.lo[r]) {  // H at the left edge is the row max
                        R.trow = i0 + r;
                        R.tleft = true;
                        R.tclamp = S.lo[r] <= 1;
                    } else if (S.hi[r] < n && S.Hl[r] == rowHp) {
                        R.trow = i0 + r;
                        R.tleft = false;
                        R.tclamp = S.hi[r] >= n;
                    }
                }
                if (rowHp > R.bestHp) {
                    R.bestHp = rowHp;
                    R.best_i = i0 + r;
                    R.best_j = argj;
                }
            }
        }
        plo = lo7;
        phi = S.hi[STRIP - 1];
    }
    return R;
}

__device__ __forceinline__ bool neutral_col(uint32_t q, uint32_t r) {
    return q < 4 && r < 4 && (q == r || (r == 0 && q == 2) || (r == 3 && q == 1));
}

// Step kinds recorded by the first traceback walk (4 bits each) so the second
// walk replays from registers/local memory instead of re-reading the
// traceback words: M with a match / mismatch / zero (editing-exempt) score,
// I or D opening a gap run (walk order), I or D extending it.
enum : int { K_MM = 0, K_MX = 1, K_MZ = 2, K_IO = 3, K_IE = 4, K_DO = 5, K_DE = 6 };
constexpr int REC_WORDS = 64;  // 512 recorded steps; longer walks re-walk
constexpr int RUNS_LOCAL = 16;  // CIGAR runs kept in the thread's own list

__device__ __forceinline__ int kind_op(int k) { return k < 3 ? ESP_OP_M : (k < 5 ? ESP_OP_I : ESP_OP_D); }

// One traceback walk over the packed bits (extend.rs:884-930): state machine
// H/E/F from (best_i, best_j), stopping at i <= 0, j <= 0, outside the row
// window, or on an H START cell.  Word loads are cached and the word of the
// next column is prefetched (most steps move one column left in the strip);
// the read and window codes at the walk's position ride in shift registers
// that move with it (reloaded 16 bases at a time), and each step's kind and
// next state are chosen by selects, so that the lanes' walks, which take
// different kinds of steps, do not split on branches.
template <int TBS>
struct Walker {
    const Geo &g;
    const uint32_t *tb;
    int sw;
    const Seq &read;
    const Seq &win;
    const GotohConst &K;
    int i, j, state;
    int cs, cclo;          // current strip and its first column
    int pdelta, pmin;      // word index offset of (i-8, j-8) and the first j it exists for
    int ck, nk;            // cached / prefetched word index
    uint32_t cw, nw;

    __device__ Walker(const Geo &g_, const uint32_t *tb_, int sw_, const Seq &r_, const Seq &w_,
                      const GotohConst &K_, int bi, int bj)
        : g(g_), tb(tb_), sw(sw_), read(r_), win(w_), K(K_), i(bi), j(bj), state(0), cs(-1),
          cclo(0), pdelta(0), pmin(0x7fffffff), ck(-1), nk(-1), cw(0), nw(0) {}

    // codes of read position i-1 and window position j-1 at bits 1:0 (N
    // flag at bit 0 of rnb / wnb); rleft / wleft = positions below still
    // in the register (< 0: reload)
    uint32_t rv = 0, wv = 0, rnb = 0, wnb = 0;
    int rleft = -1, wleft = -1;
    __device__ __forceinline__ void rfill() {
        const int q = i - 1, q0 = q >= 15 ? q - 15 : 0, k = q - q0;
        rv = load16(read.arena, read.pos + (uint64_t)q0) >> (30 - 2 * k);
        rnb = read.cnt ? nmask16(read.iv, read.cnt, q0) >> (31 - k) : 0u;
        rleft = k;
    }
    __device__ __forceinline__ void wfill() {
        const int q = j - 1, q0 = q >= 15 ? q - 15 : 0, k = q - q0;
        wv = load16(win.arena, win.pos + (uint64_t)q0) >> (30 - 2 * k);
        wnb = win.cnt ? nmask16(win.iv, win.cnt, q0) >> (31 - k) : 0u;
        wleft = k;
    }
    __device__ __forceinline__ void idec() {
        i--;
        rv >>= 2;
        rnb >>= 1;
        rleft--;
    }
    __device__ __forceinline__ void jdec() {
        j--;
        wv >>= 2;
        wnb >>= 1;
        wleft--;
    }

    // Take one step; returns false when the walk stops.  `kind` is the step.
    __device__ __forceinline__ bool step(int &kind) {
        if (i <= 0 || j <= 0) return false;
        if (j < g.lo(i) || j > g.hi(i)) return false;
        int s = (i - 1) >> 3, r = (i - 1) & 7;
        if (s != cs) {
            cs = s;
            cclo = g.lo(s * STRIP + 1);
            if (TBS == 32 && s > 0) {  // (i-8, j-8) lies in strip s-1, row r
                const int pclo = g.lo((s - 1) * STRIP + 1);
                pdelta = cclo - pclo - sw - 8;
                pmin = pclo + 8;
            }
        }
        // word indices fit 32 bits: a slot holds at most 4,096 strips of
        // 32,767 columns
        const int idx = s * sw + (j - cclo);
        uint32_t w;
        if (idx == ck) {
            w = cw;
        } else if (idx == nk) {
            w = nw;
        } else {
            w = tb[(size_t)(uint32_t)idx * TBS];
        }
        ck = idx;
        cw = w;
        if (j - 1 >= cclo) {  // prefetch the word one column left (same strip)
            nk = idx - 1;
            nw = tb[(size_t)(uint32_t)nk * TBS];
        } else {
            nk = -1;
        }
        // L2 prefetch of the word 8 diagonal steps ahead (the lane-interleaved
        // global traceback of the thread kernels): the walk mostly runs
        // along the diagonal, and the lines it reads have left L2 since the
        // fill wrote them
        if (TBS == 32 && s > 0 && j >= pmin) {
            const uint32_t *pa = tb + (size_t)(uint32_t)(idx + pdelta) * TBS;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(pa));
        }
        int sh = 2 * (7 - r);
        uint32_t hsrc = (w >> sh) & 3u;
        uint32_t eo = (w >> (16 + sh)) & 1u;
        uint32_t fo = (w >> (17 + sh)) & 1u;
        // the step's source: the cell's H tag in state 0, else the gap it is in
        const uint32_t eff = state == 0 ? hsrc : (state == 1 ? 1u : 0u);
        if (eff == 3u) return false;  // H_START
        if (rleft < 0) rfill();
        if (wleft < 0) wfill();
        const uint32_t q = (rnb & 1u) ? 4u : (rv & 3u), rc = (wnb & 1u) ? 4u : (wv & 3u);
        const int open = state == 0;
        const int kdiag = (int)((K.dkind >> (2 * (q * 5 + rc))) & 3u);
        const int kvert = open ? K_IO : K_IE, khor = open ? K_DO : K_DE;
        kind = eff == 2u ? kdiag : (eff == 1u ? kvert : khor);
        state = eff == 2u ? 0 : (eff == 1u ? (eo ? 0 : 1) : (fo ? 0 : 2));
        if (eff != 0u) idec();
        if (eff != 1u) jdec();
        return true;
    }
};

struct CigarOut {
    uint32_t *p;
    uint32_t cap;
    bool overflow;
    __device__ __forceinline__ void put(uint32_t idx, uint32_t v) {
        if (idx < cap) p[idx] = v;
        else overflow = true;
    }
};

// Traceback, end trimming, rebuild and neutral flanks (extend.rs:864-1068).
// TBS: word stride of the traceback (32 for the lane-interleaved scratch of
// the thread-per-pair kernel, 1 for the warp-per-pair kernel's own scratch).
template <int TBS>
__device__ void dp_finish(const GotohConst &K, const int8_t *__restrict__ lut, const Geo &g,
                          const uint32_t *tb, int sw, int m, int n, const Seq &read,
                          const Seq &win, const FillResult &F, esp_extension &o, uint32_t *cig,
                          uint32_t cap) {
    const int dtab[7] = {K.match, (int)K.lut[1], 0, K.open_ext, K.ext, K.open_ext, K.ext};
    // Walk 1 records each 8-step block of the walk: its steps' kinds (rec),
    // the prefix sum before it (pst) and its largest prefix sum (bmx), so
    // that the trim below finds its cut by blocks instead of re-walking.
    uint32_t rec[REC_WORDS];
    int pst[REC_WORDS], bmx[REC_WORDS];
    // walk 1: number of steps N, total T and trail (the walk's steps up to
    // and including its last non-positive prefix sum)
    int N = 0, P = 0, trail = 0;
    {
        Walker<TBS> W(g, tb, sw, read, win, K, F.best_i, F.best_j);
        int kind;
        uint32_t acc = 0;  // the open block's kinds, entering at the top
        int bm = INT_MIN, pb = 0;
        while (W.step(kind)) {
            P += dtab[kind];
            bm = max(bm, P);
            acc = (acc >> 4) | ((uint32_t)kind << 28);
            N++;
            if ((N & 7) == 0) {
                if ((N >> 3) <= REC_WORDS) {
                    rec[(N >> 3) - 1] = acc;
                    pst[(N >> 3) - 1] = pb;
                    bmx[(N >> 3) - 1] = bm;
                }
                bm = INT_MIN;
                pb = P;
            }
            if (P <= 0) trail = N;
        }
        if ((N & 7) && (N >> 3) < REC_WORDS) {
            rec[N >> 3] = acc >> (4 * (8 - (N & 7)));
            pst[N >> 3] = pb;
            bmx[N >> 3] = bm;
        }
    }
    const bool replay = N <= REC_WORDS * 8;
    const int T = P;
    uint32_t read_start, ref_start, read_end, ref_end;
    int score = 0;
    CigarOut co{cig, cap, false};
    uint32_t K_runs = 0;  // kept runs in walk order: rr, or from cig[2] when many
    uint32_t rr[RUNS_LOCAL];
    // A run goes to the thread's local list, so short CIGARs are written
    // once, in final order, with no global read-back, and need only their
    // final length in capacity; a long CIGAR moves the list to its slots
    // cig[2..] (and needs them: it is reversed there in place).
    auto emit = [&](uint32_t v) {
        if (K_runs < RUNS_LOCAL) {
            rr[K_runs] = v;
        } else {
            if (K_runs == RUNS_LOCAL)
                for (int k = 0; k < RUNS_LOCAL; k++) co.put(2 + k, rr[k]);
            co.put(2 + K_runs, v);
        }
        K_runs++;
    };
    int first_op = -1, last_op = -1;  // forward order first / last kept op
    if (N == 0) {
        read_start = (uint32_t)max(F.best_i, 0);
        ref_start = (uint32_t)max(F.best_j, 0);
        read_end = read_start;
        ref_end = ref_start;
    } else if (replay) {
        // With walk-order prefix sums P_t, the reference's forward lead is
        // N-1-u where u is the first index in [-1, N-2] with P_u >= T
        // (P_-1 = 0): the first block whose largest prefix sum reaches T
        // holds it (the last block always does, through P_N-1 = T, but
        // only its steps up to N-2 count).  The kept steps are walk indices
        // [trail, u] -- through N-1 when no u exists -- and lead + trail >=
        // N (the degenerate keep-the-middle case, extend.rs:956-960) is
        // exactly u < trail, or T <= 0.
        int ue = N - 1, Pue = T;
        bool degenerate = T <= 0;
        if (!degenerate) {
            const int nb = (N + 7) >> 3;
            for (int b = 0; b < nb; b++) {
                if (bmx[b] < T) continue;
                int Pb = pst[b];
                uint32_t w = rec[b];
                const int tend = min(8 * b + 7, N - 2);
                int t = 8 * b;
                for (; t <= tend; t++, w >>= 4) {
                    Pb += dtab[w & 15u];
                    if (Pb >= T) break;
                }
                if (t <= tend) {
                    ue = t;
                    Pue = Pb;
                    degenerate = t < trail;
                }
                break;
            }
        }
        if (degenerate) {  // the middle step t* = N-1-N/2 alone
            const int tstar = N - 1 - N / 2;
            int i = F.best_i, j = F.best_j, op = 0, d = 0;
            for (int t = 0; t <= tstar; t++) {
                const int kind = (int)((rec[t >> 3] >> (4 * (t & 7))) & 15u);
                op = kind_op(kind);
                d = dtab[kind];
                if (t == tstar) break;
                if (op != ESP_OP_D) i--;
                if (op != ESP_OP_I) j--;
            }
            read_end = (uint32_t)i;
            ref_end = (uint32_t)j;
            read_start = (uint32_t)(op != ESP_OP_D ? i - 1 : i);
            ref_start = (uint32_t)(op != ESP_OP_I ? j - 1 : j);
            score = d;
            emit((1u << 4) | (uint32_t)op);
            first_op = last_op = op;
        } else {
            // the cell the walk stood on before step `trail` and the prefix
            // sum there, from the record
            int tr_i = F.best_i, tr_j = F.best_j, ptrail = 0;
            for (int t = 0; t < trail; t++) {
                const int kind = (int)((rec[t >> 3] >> (4 * (t & 7))) & 15u);
                const int op = kind_op(kind);
                ptrail += dtab[kind];
                if (op != ESP_OP_D) tr_i--;
                if (op != ESP_OP_I) tr_j--;
            }
            // runs of steps [trail, ue] in walk order; the kept region ends
            // (forward order) where the walk stood before step `trail`
            read_end = (uint32_t)tr_i;
            ref_end = (uint32_t)tr_j;
            uint32_t w = rec[trail >> 3] >> (4 * (trail & 7));
            last_op = kind_op((int)(w & 15u));
            int cur_op = last_op;
            uint32_t cur_len = 0, di = 0, dj = 0;
            for (int t = trail; t <= ue; t++) {
                if ((t & 7) == 0) w = rec[t >> 3];
                const int op = kind_op((int)(w & 15u));
                w >>= 4;
                if (op != cur_op) {
                    emit((cur_len << 4) | (uint32_t)cur_op);
                    if (cur_op != ESP_OP_D) di += cur_len;
                    if (cur_op != ESP_OP_I) dj += cur_len;
                    cur_op = op;
                    cur_len = 0;
                }
                cur_len++;
            }
            emit((cur_len << 4) | (uint32_t)cur_op);
            if (cur_op != ESP_OP_D) di += cur_len;
            if (cur_op != ESP_OP_I) dj += cur_len;
            first_op = cur_op;
            read_start = read_end - di;
            ref_start = ref_end - dj;
            score = Pue - ptrail;
        }
    } else {
        // Walks longer than the record: walk 2 re-walks the traceback,
        // finding u (as above) on the way.  Step t* (the middle step) is
        // captured in case the degenerate case comes up.
        bool degenerate = (T <= 0);  // u = -1
        const int tstar = N - 1 - N / 2;
        Walker<TBS> W(g, tb, sw, read, win, K, F.best_i, F.best_j);
        int i = F.best_i, j = F.best_j;
        int pos_acc = 0;
        bool found = false;
        int cur_op = -1;
        uint32_t cur_len = 0;
        read_end = ref_end = read_start = ref_start = 0;
        int ts_ib = 0, ts_jb = 0, ts_ia = 0, ts_ja = 0, ts_op = 0, ts_d = 0;
        bool done = false;
        for (int t = 0; t < N && !done; t++) {
            int i_before = i, j_before = j;
            int kind;
            W.step(kind);
            int op = kind_op(kind), d = dtab[kind];
            if (op != ESP_OP_D) i--;
            if (op != ESP_OP_I) j--;
            if (t == tstar) {
                ts_ib = i_before;
                ts_jb = j_before;
                ts_ia = i;
                ts_ja = j;
                ts_op = op;
                ts_d = d;
            }
            pos_acc += d;
            if (!degenerate && !found && t <= N - 2 && pos_acc >= T) {
                found = true;
                if (t < trail) degenerate = true;  // nothing emitted yet
            }
            if (degenerate) {
                if (t >= tstar) done = true;
                continue;
            }
            if (t >= trail) {
                if (t == trail) {
                    read_end = (uint32_t)i_before;
                    ref_end = (uint32_t)j_before;
                    last_op = op;
                }
                score += d;
                if (op == cur_op) {
                    cur_len++;
                } else {
                    if (cur_op >= 0) emit((cur_len << 4) | (uint32_t)cur_op);
                    cur_op = op;
                    cur_len = 1;
                }
                first_op = op;
                if (found) {  // t == u_min: the kept region starts here
                    read_start = (uint32_t)i;
                    ref_start = (uint32_t)j;
                    done = true;
                }
            }
        }
        if (degenerate) {
            read_end = (uint32_t)ts_ib;
            ref_end = (uint32_t)ts_jb;
            read_start = (uint32_t)ts_ia;
            ref_start = (uint32_t)ts_ja;
            score = ts_d;
            K_runs = 0;
            emit((1u << 4) | (uint32_t)ts_op);
            first_op = last_op = ts_op;
        } else {
            if (cur_op >= 0) emit((cur_len << 4) | (uint32_t)cur_op);
            if (!found) {  // lead = 0: kept through the last step
                read_start = (uint32_t)i;
                ref_start = (uint32_t)j;
            }
        }
    }
    // reverse the kept runs into forward order (a long CIGAR's, in place)
    if (!co.overflow && K_runs > RUNS_LOCAL) {
        for (uint32_t a = 0, b = K_runs ? K_runs - 1 : 0; a < b; a++, b--) {
            uint32_t t = cig[2 + a];
            cig[2 + a] = cig[2 + b];
            cig[2 + b] = t;
        }
    }
    // neutral flanks (extend.rs:991-1049)
    uint32_t nl = 0, nr = 0;
    if (score > 0) {
        int delta = 0;
        uint32_t lim = min(read_start, ref_start);
        for (uint32_t k = 1; k <= lim; k++) {
            uint32_t q = read.code((int64_t)read_start - k), r = win.code((int64_t)ref_start - k);
            if (!neutral_col(q, r)) break;
            delta += lut[q * 5 + r];
            if (delta == 0) nl = k;
        }
        delta = 0;
        uint32_t av = min((uint32_t)m - read_end, (uint32_t)n - ref_end);
        for (uint32_t k = 0; k < av; k++) {
            uint32_t q = read.code((int64_t)read_end + k), r = win.code((int64_t)ref_end + k);
            if (!neutral_col(q, r)) break;
            delta += lut[q * 5 + r];
            if (delta == 0) nr = k + 1;
        }
        read_start -= nl;
        ref_start -= nl;
        read_end += nr;
    }
    // final CIGAR: S, M(neutral), kept runs, M(neutral), S (push_op merging)
    uint32_t total = K_runs;
    if (nl > 0 && first_op != ESP_OP_M) total++;
    if (nr > 0 && last_op != ESP_OP_M) total++;
    if (read_start > 0) total++;
    if (read_end < (uint32_t)m) total++;
    if (!co.overflow && total <= cap) {
        uint32_t w = 0;
        int prev = -1;
        auto push = [&](uint32_t op, uint32_t len) {
            if ((int)op == prev) {
                cig[w - 1] += len << 4;
            } else {
                cig[w++] = (len << 4) | op;
                prev = (int)op;
            }
        };
        if (read_start > 0) push(ESP_OP_S, read_start);
        if (nl > 0) push(ESP_OP_M, nl);
        for (uint32_t k = 0; k < K_runs; k++) {
            uint32_t v = K_runs <= RUNS_LOCAL ? rr[K_runs - 1 - k] : cig[2 + k];
            push(v & 15u, v >> 4);
        }
        if (nr > 0) push(ESP_OP_M, nr);
        if (read_end < (uint32_t)m) push(ESP_OP_S, (uint32_t)m - read_end);
        o.status = ESP_OK;
    } else {
        o.status = ESP_ECAP;
    }
    o.n_ops = total;
    o.read_start = read_start;
    o.read_end = read_end;
    o.ref_start = ref_start;
    o.score = score;
}

// A validated pair: geometry for the job's mode, sequences, output slot and
// the result record being built.
struct PairSetup {
    int m, n, sw;
    bool full;
    Geo g;
    Seq read, win;
    uint32_t *cig;
    esp_extension o;
};

// Validate pair pi and resolve its band geometry (extend.rs:392-428 for the
// extend_hint attempts).  Returns true when a DP is needed; otherwise the
// result (empty extension, or a refusal) has been written when `write`.
__device__ __forceinline__ bool setup_pair(const GotohJob &job, const GotohConst &K, uint32_t pi,
                                           uint64_t tb_cap, uint64_t rb_cap, bool write,
                                           PairSetup &S) {
    if (pi >= job.n_pairs) return false;  // corrupt work list: never index past the batch
    esp_pair P = job.pairs[pi];
    int m = (int)P.read_len, n = (int)P.win_len;
    esp_extension &o = S.o;
    o.read_start = o.read_end = o.ref_start = 0;
    o.score = 0;
    o.n_ops = 0;
    o.touch_row = 0;
    o.touched = o.touch_left = o.touch_clamped = 0;
    o.escalated = job.mode == 2 ? 1 : 0;
    o.status = ESP_OK;
    S.cig = job.cigar + (uint64_t)pi * job.cigar_stride;
    if (m == 0 || n == 0) {  // extend.rs:430-442 empty_extension
        if (m > 0) {
            o.n_ops = 1;
            if (job.cigar_stride >= 1) {
                if (write) S.cig[0] = ((uint32_t)m << 4) | ESP_OP_S;
            } else {
                o.status = ESP_ECAP;
            }
        }
        if (write) job.out[pi] = o;
        return false;
    }
    Geo g;
    bool full;
    if (job.mode == 0) {
        full = P.band_half < 0;
        g.off = full ? 0 : P.band_offset;
        g.half = full ? n : P.band_half;
    } else if (job.mode == 1) {
        full = 30 >= n;  // INITIAL_BAND >= window: full matrix, accepted directly
        g.off = full ? 0 : P.band_offset;
        g.half = full ? n : 30;
    } else {
        full = true;
        g.off = 0;
        g.half = n;
    }
    g.n = n;
    int sw = full ? n : min(2 * g.half + STRIP, n);
    uint64_t need_tb = (uint64_t)((m + STRIP - 1) / STRIP) * (uint64_t)sw;
    uint64_t need_rb = (uint64_t)sw;
    const uint8_t *warena = job.win_arena ? job.win_arena : job.arena;
    const uint64_t wbases = job.win_arena ? job.win_arena_bases : job.arena_bases;
    const bool outside = (uint64_t)P.n_first + P.n_read + P.n_win > job.n_iv_count ||
                         P.read_pos + (uint64_t)m > job.arena_bases ||
                         P.win_pos + (uint64_t)n > wbases || m > 32767 || n > 32767;
    if (!outside && m > K.max_m && !job.wide && job.wide_list) {
        // scores may leave the int16 domain: the wide kernel runs this pair
        if (write) job.wide_list[atomicAdd(job.wide_count, 1u)] = pi;
        return false;
    }
    if (need_tb > tb_cap || need_rb > rb_cap || outside || (m > K.max_m && !job.wide)) {
        // scratch sized too small by the host, or the pair lies outside its
        // tables: refuse, never overrun
        o.status = ESP_EINVAL;
        if (write) job.out[pi] = o;
        return false;
    }
    const esp_n_interval *iv = job.n_iv + P.n_first;
    S.read = Seq{job.arena, P.read_pos, iv, P.n_read};
    S.win = Seq{warena, P.win_pos, iv + P.n_read, P.n_win};
    S.m = m;
    S.n = n;
    S.sw = sw;
    S.full = full;
    S.g = g;
    return true;
}

// Traceback, CIGAR, TouchRec, extend_hint escalation (extend.rs:421-426),
// then the result record.  Returns whether attempt 1 escalates; the pair is
// appended to the escalation list when `queue` (the wide kernel runs its
// second attempt itself).
template <int TBS>
__device__ __forceinline__ bool finish_pair(const GotohJob &job, const GotohConst &K,
                                            const int8_t *__restrict__ lut, uint32_t pi,
                                            PairSetup &S, const FillResult &F,
                                            const uint32_t *tb, bool queue = true) {
    esp_extension &o = S.o;
    dp_finish<TBS>(K, lut, S.g, tb, S.sw, S.m, S.n, S.read, S.win, F, o, S.cig,
                   job.cigar_stride);
    if (F.trow) {
        o.touched = 1;
        o.touch_row = F.trow;
        o.touch_left = F.tleft ? 1 : 0;
        o.touch_clamped = F.tclamp ? 1 : 0;
    }
    bool esc = false;
    if (job.mode == 1 && !S.full) {
        // escalate on a band-edge touch or < 85% of perfect
        int perfect = S.m * K.match;
        if (F.trow != 0 || o.score * 20 < perfect * 17) {
            if (queue) job.esc_list[atomicAdd(job.esc_count, 1u)] = pi;
            o.escalated = 1;
            esc = true;
        }
    }
    job.out[pi] = o;
    return esc;
}

__device__ void process_pair(const GotohJob &job, const GotohConst &K,
                             const uint32_t *__restrict__ s_lut, const int8_t *__restrict__ lut,
                             uint32_t pi, uint32_t *tb, uint32_t *rb) {
    PairSetup S;
    if (!setup_pair(job, K, pi, job.tb_words, job.rb_words, true, S)) return;
    FillResult F = S.win.cnt ? dp_fill<true>(K, s_lut, S.m, S.n, S.g, S.read, S.win, tb, S.sw, rb)
                             : dp_fill<false>(K, s_lut, S.m, S.n, S.g, S.read, S.win, tb, S.sw, rb);
    finish_pair<32>(job, K, lut, pi, S, F, tb);
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) gotoh_kernel(GotohJob job, GotohConst K) {
    __shared__ uint32_t s_lut[10];
    __shared__ int8_t s_lut25[32];
    if (threadIdx.x == 0) {  // static indices keep the parameter block out of local memory
#pragma unroll
        for (int k = 0; k < 10; k++) s_lut[k] = K.lut4[k >> 1][k & 1];
#pragma unroll
        for (int k = 0; k < 25; k++) s_lut25[k] = K.lut[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t warp_slot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t *tb = job.tb + warp_slot * job.tb_words * 32 + lane;
    uint32_t *rb = job.rb + warp_slot * job.rb_words * 32 + lane;
    uint64_t b0 = 0, total = job.list_count ? (uint64_t)(*job.list_count) : job.n_pairs;
    if (job.range) {  // one length class of the binned list
        b0 = job.range[0];
        total = job.range[1] > job.range[0] ? job.range[1] - job.range[0] : 0;
    }
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd((unsigned long long *)job.queue, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        uint64_t k = base + lane;
        if (k < total) {
            uint32_t pi = job.list ? job.list[b0 + k] : (uint32_t)(b0 + k);
            process_pair(job, K, s_lut, s_lut25, pi, tb, rb);
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-per-pair DP (the per-call drop-in and small batches).  One pair's
// strips are spread over the lanes of a warp (lane s owns rows 8s+1..8s+8 of
// the current 32-strip pass) and swept as a wavefront: at step t lane s
// evaluates column j = t - s, receiving the bottom row (H, E) of lane s-1 at
// the same column by a warp shuffle (lane s-1 produced it one step earlier)
// and keeping the previous step's value as its diagonal.  Idle or
// out-of-window lanes publish H = 0, E = NEG -- what the thread-per-pair
// kernel's row buffer presents outside the previous strip's window -- so
// every cell, traceback word, row maximum and touch is the same as there.
// A pass of 32 strips hands its last row to the next pass through the row
// buffer.  Lane 0 then walks the traceback.  Scratch is the warp's own
// (word stride 1).
// ---------------------------------------------------------------------------

// WIDE = false: H and E of a row cross lanes and passes packed as int16
// halves of one word (the int16 domain); WIDE = true: as two int32 words
// (the row buffer then holds 2 words per column).
template <bool WIDE>
__device__ FillResult warp_fill(const GotohConst &K, const uint32_t *__restrict__ s_lut,
                                const PairSetup &P, uint32_t *tb, uint32_t *rb, int lane) {
    const int m = P.m, n = P.n, sw = P.sw;
    const Geo &g = P.g;
    const uint32_t ABSENT = __byte_perm(2u, (uint32_t)NEG4, 0x5410);  // H = 0, E = NEG
    FillResult R;
    R.bestHp = 2;
    R.best_i = R.best_j = 0;
    R.trow = 0;
    R.tleft = R.tclamp = false;
    const int nstrips = (m + STRIP - 1) / STRIP;
    for (int base = 0; base < nstrips; base += 32) {
        const int s = base + lane;
        const bool act = s < nstrips;
        const int i0 = s * STRIP + 1;
        const int nact = act ? min(STRIP, m - i0 + 1) : 0;
        StripT<WIDE> S;
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            S.lo[r] = g.lo(i0 + r);
            S.hi[r] = g.hi(i0 + r);
            S.Hl[r] = 2;
            S.Fl[r] = NEG4;
            S.rk[r] = -1;
        }
        const int clo = S.lo[0];
        const int chi = act ? g.hi(i0 + nact - 1) : 0;
        const int lo7 = S.lo[STRIP - 1];
        if (act) {
            uint32_t rw = load16(P.read.arena, P.read.pos + (uint64_t)(i0 - 1));
            uint32_t rn = P.read.cnt ? nmask16(P.read.iv, P.read.cnt, i0 - 1) : 0u;
#pragma unroll
            for (int r = 0; r < STRIP; r++) {
                uint32_t c = (rw >> (30 - 2 * r)) & 3u;
                if ((rn >> (31 - r)) & 1u) c = 4;
                S.l0[r] = s_lut[2 * c];
                S.l1[r] = s_lut[2 * c + 1];
            }
        }
        // the previous pass's last strip left its bottom row in rb, columns
        // [plo, phi] of row 8*base
        const int plo = base ? g.lo(base * STRIP) : 0, phi = base ? g.hi(base * STRIP) : -1;
        int t0 = act ? clo + lane : 0x7fffffff, t1 = act ? chi + lane : -1;
        t0 = __reduce_min_sync(0xffffffffu, t0);
        t1 = __reduce_max_sync(0xffffffffu, t1);
        // bottom row published at the end of a step: packed (int16) or H / E (int32)
        uint32_t pub = ABSENT;
        int pubH = 2, pubE = NEG4;
        int diag = 2;           // H of the row above at the previous column
        if (lane == 0 && base && clo - 1 >= plo && clo - 1 <= phi)
            diag = WIDE ? (int)rb[2 * (clo - 1 - plo)] : (int)(rb[clo - 1 - plo] & 0xffffu);
        uint32_t *tbs = tb + (size_t)s * sw;
        const bool handoff = lane == 31 && s + 1 < nstrips;
        int cw_at = -1000000;  // first window position of the cached code word
        uint32_t cw = 0, cn = 0;
        int nx_at = -1000000;  // the word after it, loaded one word ahead
        uint32_t nx = 0, nxn = 0;
        for (int t = t0; t <= t1; t++) {
            const int j = t - lane;
            int inH, inE;
            if (WIDE) {
                inH = __shfl_up_sync(0xffffffffu, pubH, 1);
                inE = __shfl_up_sync(0xffffffffu, pubE, 1);
                if (lane == 0) {
                    const bool have = base && j >= plo && j <= phi;
                    inH = have ? (int)rb[2 * (j - plo)] : 2;
                    inE = have ? (int)rb[2 * (j - plo) + 1] : NEG4;
                }
            } else {
                uint32_t in = __shfl_up_sync(0xffffffffu, pub, 1);
                if (lane == 0) in = (base && j >= plo && j <= phi) ? rb[j - plo] : ABSENT;
                inH = (int)(in & 0xffffu);
                inE = ((int)in) >> 16;
            }
            int outH = 2, outE = NEG4;
            if (act && j >= clo && j <= chi) {
                // window codes 16 at a time, each word loaded while the
                // one before is in use: a load that a lane waits for stalls
                // the whole wavefront, and the lanes reach their word
                // boundaries at different steps
                if (j - 1 >= cw_at + 16) {
                    if (j - 1 == nx_at) {
                        cw = nx;
                        cn = nxn;
                    } else {
                        cw = load16(P.win.arena, P.win.pos + (uint64_t)(j - 1));
                        cn = P.win.cnt ? nmask16(P.win.iv, P.win.cnt, j - 1) : 0u;
                    }
                    cw_at = j - 1;
                    nx_at = cw_at + 16;
                    if (nx_at < n) {
                        nx = load16(P.win.arena, P.win.pos + (uint64_t)nx_at);
                        nxn = P.win.cnt ? nmask16(P.win.iv, P.win.cnt, nx_at) : 0u;
                    }
                }
                const int sh = j - 1 - cw_at;
                uint32_t code = ((cn >> (31 - sh)) & 1u) ? 4u : ((cw >> (30 - 2 * sh)) & 3u);
                uint32_t sel = code * 0x1111u + 0x8880u;
                int upH = inH, upE = inE;
                uint32_t word = dp_column<1, WIDE>(S, K, j, sel, 32767u - (uint32_t)j, upH, upE,
                                                   diag);
                tbs[j - clo] = word;
                outH = upH;
                outE = upE;
                if (handoff && j >= lo7) {
                    if (WIDE) {
                        rb[2 * (j - lo7)] = (uint32_t)upH;
                        rb[2 * (j - lo7) + 1] = (uint32_t)upE;
                    } else {
                        rb[j - lo7] = __byte_perm((uint32_t)upH, (uint32_t)upE, 0x5410);
                    }
                }
            }
            diag = inH;
            if (WIDE) {
                pubH = outH;
                pubE = outE;
            } else {
                pub = __byte_perm((uint32_t)outH, (uint32_t)outE, 0x5410);
            }
        }
        __syncwarp();
        // this lane's rows, in row order (extend.rs:795-827)
        int bHp = -1, bi = 0, bj = 0, trow = 0;
        bool tleft = false, tclamp = false;
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            if (r < nact) {
                int rowHp = (int)(S.rk[r] >> 15);
                int argj = 32767 - (int)(S.rk[r] & 32767);
                if (trow == 0) {
                    if (argj == S.lo[r]) {
                        trow = i0 + r;
                        tleft = true;
                        tclamp = S.lo[r] <= 1;
                    } else if (S.hi[r] < n && S.Hl[r] == rowHp) {
                        trow = i0 + r;
                        tleft = false;
                        tclamp = S.hi[r] >= n;
                    }
                }
                if (rowHp > bHp) {
                    bHp = rowHp;
                    bi = i0 + r;
                    bj = argj;
                }
            }
        }
        // merge lanes in row order: the first strictly larger maximum wins,
        // the first touching row wins
        const int mx = __reduce_max_sync(0xffffffffu, bHp);
        const int wl = __ffs(__ballot_sync(0xffffffffu, bHp == mx)) - 1;
        const int wi = __shfl_sync(0xffffffffu, bi, wl), wj = __shfl_sync(0xffffffffu, bj, wl);
        if (mx > R.bestHp) {
            R.bestHp = mx;
            R.best_i = wi;
            R.best_j = wj;
        }
        const uint32_t tm = __ballot_sync(0xffffffffu, trow != 0);
        if (R.trow == 0 && tm) {
            const int tl = __ffs(tm) - 1;
            R.trow = __shfl_sync(0xffffffffu, trow, tl);
            R.tleft = __shfl_sync(0xffffffffu, (int)tleft, tl) != 0;
            R.tclamp = __shfl_sync(0xffffffffu, (int)tclamp, tl) != 0;
        }
    }
    return R;
}

__global__ void __launch_bounds__(128) gotoh_warp_kernel(GotohJob job, GotohConst K) {
    __shared__ uint32_t s_lut[10];
    __shared__ int8_t s_lut25[32];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) s_lut[k] = K.lut4[k >> 1][k & 1];
#pragma unroll
        for (int k = 0; k < 25; k++) s_lut25[k] = K.lut[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t warp_slot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t *tb = job.tb + warp_slot * (job.tb_words + job.rb_words);
    uint32_t *rb = tb + job.tb_words;
    const uint64_t total = job.list_count ? (uint64_t)(*job.list_count) : job.n_pairs;
    for (uint64_t k = warp_slot; k < total; k += n_warps) {
        const uint32_t pi = job.list ? job.list[k] : (uint32_t)k;
        PairSetup S;
        if (!setup_pair(job, K, pi, job.tb_words, job.rb_words, lane == 0, S)) continue;
        FillResult F = warp_fill<false>(K, s_lut, S, tb, rb, lane);
        __syncwarp();  // traceback words of every lane are visible to lane 0
        if (lane == 0) finish_pair<1>(job, K, s_lut25, pi, S, F, tb);
        __syncwarp();
    }
}

cudaError_t launch_gotoh_warp(const GotohJob &job, const GotohConst &k, int warps,
                              cudaStream_t st) {
    int grid = (warps + 3) / 4;
    gotoh_warp_kernel<<<grid, 128, 0, st>>>(job, k);
    return cudaGetLastError();
}

// Pairs outside the int16 domain (reads longer than GotohConst::max_m), one
// warp per pair with int32 H / E / F and 64-bit row-max keys, otherwise the
// warp-per-pair fill and the same traceback: the same cells, words, maxima,
// touches and CIGARs as the reference's i32 flavour of run_band
// (extend.rs:462-528).  In hint mode the warp runs extend_hint's second
// attempt itself when the first escalates (extend.rs:421-426).
__global__ void __launch_bounds__(128) gotoh_wide_kernel(GotohJob job, GotohConst K) {
    __shared__ uint32_t s_lut[10];
    __shared__ int8_t s_lut25[32];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) s_lut[k] = K.lut4[k >> 1][k & 1];
#pragma unroll
        for (int k = 0; k < 25; k++) s_lut25[k] = K.lut[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t warp_slot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t *tb = job.tb + warp_slot * (job.tb_words + 2 * job.rb_words);
    uint32_t *rb = tb + job.tb_words;
    const uint64_t total = *job.list_count;
    for (uint64_t k = warp_slot; k < total; k += n_warps) {
        const uint32_t pi = job.list[k];
        PairSetup S;
        if (!setup_pair(job, K, pi, job.tb_words, job.rb_words, lane == 0, S)) continue;
        FillResult F = warp_fill<true>(K, s_lut, S, tb, rb, lane);
        __syncwarp();
        int esc = 0;
        if (lane == 0) esc = finish_pair<1>(job, K, s_lut25, pi, S, F, tb, false) ? 1 : 0;
        esc = __shfl_sync(0xffffffffu, esc, 0);
        __syncwarp();
        if (!esc) continue;
        GotohJob j2 = job;
        j2.mode = 2;
        if (!setup_pair(j2, K, pi, job.tb_words, job.rb_words, lane == 0, S)) continue;
        F = warp_fill<true>(K, s_lut, S, tb, rb, lane);
        __syncwarp();
        if (lane == 0) finish_pair<1>(j2, K, s_lut25, pi, S, F, tb, false);
        __syncwarp();
    }
}

cudaError_t launch_gotoh_wide(const GotohJob &job, const GotohConst &k, int warps,
                              cudaStream_t st) {
    GotohJob j = job;
    j.wide = 1;
    int grid = (warps + 3) / 4;
    gotoh_wide_kernel<<<grid, 128, 0, st>>>(j, k);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Two pairs per thread in 16x2 SIMD lanes.  Two pairs with identical band
// geometry and N-free windows share one thread: every register holds the
// scaled key of pair A in its low half and of pair B in its high half, and
// the half-word operations (add-max, 3-way max) evaluate both cells at once
// with the arithmetic above (values stay inside int16: H <= 8191 by the
// score-range rule, gap keys >= -16384 - 4*ext).  Substitution scores of
// both cells come from one PRMT over the two rows' LUT words.  The traceback
// words, row maxima and touches of each pair are exactly those of the
// thread-per-pair kernel, and each pair's traceback is walked by the same
// code (its words at stride 32, pair B's region after pair A's).
// ---------------------------------------------------------------------------

constexpr uint32_t NEG2 = 0xC000C000u;   // E/F sentinel (-16384) in both halves
constexpr uint32_t VNEG2 = 0x80008000u;  // -32768: max against it is a plain add
constexpr uint32_t KEEP2 = 0xFFFCFFFCu;

struct Strip2 {
    uint32_t Hl[STRIP], Fl[STRIP], rmax[STRIP];
    uint32_t la[STRIP], lb[STRIP];
    uint32_t arg[STRIP];   // first column of the row maximum: pair A low half, B high
    uint32_t lohi[STRIP];  // row window: first column low half, last column high half
};

__device__ __forceinline__ uint32_t prmt(uint32_t lo, uint32_t hi, uint32_t sel) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(sel));
    return r;
}

// Row maximum and its first column for both lanes.  Hp and the running max
// are in [0, 32766], so old + 0x8000 - Hp per half neither carries nor
// borrows across halves and its bit 15 is set exactly when old >= Hp; PRMT's
// sign-replicate mode spreads that bit into a keep mask per half.
__device__ __forceinline__ void row_max2(uint32_t &rmax, uint32_t &arg, uint32_t Hp, uint32_t jj) {
    uint32_t t = rmax + 0x80008000u - Hp;
    uint32_t keep = prmt(t, 0u, 0xBB99u);
    rmax = (rmax & keep) | (Hp & ~keep);
    arg = (arg & keep) | (jj & ~keep);
}

template <int MASK>
__device__ __forceinline__ void dp_column2(Strip2 &S, const uint32_t oe1, const uint32_t oe4,
                                           const uint32_t ex4, int j, uint32_t sel, uint32_t &upH,
                                           uint32_t &upE, uint32_t diag, uint32_t &wa,
                                           uint32_t &wb) {
    wa = 0;
    wb = 0;
    uint32_t d = diag;
    const uint32_t jj = (uint32_t)j * 0x10001u;
#pragma unroll
    for (int r = 0; r < STRIP; r++) {
        uint32_t left = S.Hl[r];
        uint32_t kE = __viaddmax_s16x2(upE, ex4, __viaddmax_s16x2(upH, oe1, VNEG2));
        uint32_t kF = __viaddmax_s16x2(S.Fl[r], ex4, __viaddmax_s16x2(left, oe4, VNEG2));
        // tags by adds and flags by one LOP3 as in dp_column: every half's
        // result is in [0, 3] (E4 + 1 cannot carry: E4's low bits are 0), so
        // the packed 32-bit adds are exact per half
        uint32_t E4 = and_u32(kE, KEEP2);
        uint32_t F4 = and_u32(kF, KEEP2);
        uint32_t kd = __viaddmax_s16x2(d, prmt(S.la[r], S.lb[r], sel), 0x00030003u);
        uint32_t key = __vimax3_s16x2(kd, E4 + 0x00010001u, F4);
        uint32_t Hp = and_or_u32(key, KEEP2, 0x00020002u);
        wa = mad_u32(wa, 4u, key - Hp + 0x00020002u);
        wb = mad_u32(wb, 4u, or_and_u32(kE, kF, 0x00030003u));
        if (MASK) {  // out-of-window cells: as in dp_column
            const int lo = (int)(S.lohi[r] & 0xffffu), hi = (int)(S.lohi[r] >> 16);
            const bool in = (j >= lo) & (j <= hi);
            if (in) {
                row_max2(S.rmax[r], S.arg[r], Hp, jj);
                S.Hl[r] = Hp;
                S.Fl[r] = F4;
            }
            upH = in ? Hp : 0x00020002u;
            upE = in ? E4 : NEG2;
        } else {
            row_max2(S.rmax[r], S.arg[r], Hp, jj);
            S.Hl[r] = Hp;
            S.Fl[r] = F4;
            upH = Hp;
            upE = E4;
        }
        d = left;
    }
}

// Columns [a, b] for both pairs; rb holds (H, E) of both pairs per column
// (one uint2 per lane and column).
template <int MASK, bool CHECK>
__device__ __forceinline__ void dp_cols2(Strip2 &S, const uint32_t oe1, const uint32_t oe4,
                                         const uint32_t ex4, int a, int b, uint32_t &diag,
                                         const uint8_t *warena, uint64_t wposA, uint64_t wposB,
                                         uint2 *rb, int plo,
                                         int phi, int lo7, uint32_t *tbA, uint32_t *tbB) {
    uint2 *rbr = rb + (size_t)(a - plo) * 32;
    uint2 wn0 = make_uint2(0u, 0u), wn1 = make_uint2(0u, 0u);
    if (!CHECK) {  // interior: the row above two columns ahead
        wn0 = rbr[0];
        if (a + 1 <= b) wn1 = rbr[32];
    }
    for (int j = a; j <= b;) {
        uint32_t cwA = load16(warena, wposA + (uint64_t)(j - 1));
        uint32_t cwB = load16(warena, wposB + (uint64_t)(j - 1));
        int cnt = min(16, b - j + 1);
#pragma unroll 1
        for (int k = 0; k < cnt; k++, j++) {
            uint32_t sel = (cwA >> 30) * 0x11u + (cwB >> 30) * 0x1100u + 0xC480u;
            cwA <<= 2;
            cwB <<= 2;
            uint2 w = make_uint2(0x00020002u, NEG2);
            if (CHECK) {
                if (j <= phi) w = *rbr;
            } else {
                w = wn0;
                wn0 = wn1;
                if (j + 2 <= b) wn1 = rbr[64];
            }
            uint32_t upH = w.x, upE = w.y;
            uint32_t wa, wb;
            dp_column2<MASK>(S, oe1, oe4, ex4, j, sel, upH, upE, diag, wa, wb);
            diag = w.x;
            uint2 packed = make_uint2(upH, upE);
            if (CHECK) {
                if (j >= lo7) rb[(size_t)(j - lo7) * 32] = packed;
            } else {
                rbr[(ptrdiff_t)(plo - lo7) * 32] = packed;
            }
            // streaming stores: the traceback words make way in L2 for the
            // row buffer (measured +1.8 % here; the one-pair kernel's own
            // stores measured 0.8 % slower so)
            __stcs(tbA, __byte_perm(wa, wb, 0x5410));
            __stcs(tbB, __byte_perm(wa, wb, 0x7632));
            tbA += 32;
            tbB += 32;
            rbr += 32;
        }
    }
}

// Fill the DP of two pairs with identical geometry (shared g, m, n, sw).
__device__ void dp_fill2(const GotohConst &K, const uint32_t *__restrict__ s_lut, int m, int n,
                         const Geo &g, const Seq &readA, const Seq &readB, const uint8_t *warena,
                         uint64_t wposA, uint64_t wposB, uint32_t *tbA, uint32_t *tbB, int sw, uint2 *rb,
                         FillResult &FA, FillResult &FB) {
    const uint32_t oe1 = (uint32_t)(K.oe1 & 0xffff) * 0x10001u;
    const uint32_t oe4 = (uint32_t)(K.oe4 & 0xffff) * 0x10001u;
    const uint32_t ex4 = (uint32_t)(K.ex4 & 0xffff) * 0x10001u;
    // the best cell so far of both pairs, packed like the row maxima: its
    // scaled H, row and column (pair A low half, B high half); the first
    // touching row of each pair with its left / clamped flags, and bit 15 of
    // each half of open_halves while that pair has none (all in registers:
    // FA and FB are the caller's memory)
    uint32_t bestHp2 = 0x00020002u, bestI2 = 0u, bestJ2 = 0u;
    uint32_t trow2 = 0u, tflags = 0u;  // touch rows (halves); left / clamped bits 0-1 (A), 2-3 (B)
    uint32_t open_halves = 0x80008000u;
    int nstrips = (m + STRIP - 1) / STRIP;
    int plo = g.lo(1), phi = g.hi(min(STRIP, m));
    for (int k = 0; k <= phi - plo; k++) rb[(size_t)k * 32] = make_uint2(0x00020002u, NEG2);
    Strip2 S;
    for (int s = 0; s < nstrips; s++) {
        int i0 = s * STRIP + 1;
        int nact = min(STRIP, m - i0 + 1);
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            S.lohi[r] = (uint32_t)g.lo(i0 + r) | ((uint32_t)g.hi(i0 + r) << 16);
            S.Hl[r] = 0x00020002u;
            S.Fl[r] = NEG2;
            S.rmax[r] = 0u;
            S.arg[r] = 0u;
        }
        int clo = (int)(S.lohi[0] & 0xffffu);
        int chi = g.hi(i0 + nact - 1);
        int lo7 = (int)(S.lohi[STRIP - 1] & 0xffffu);
        int hi0 = (int)(S.lohi[0] >> 16);
        uint32_t rwA = load16(readA.arena, readA.pos + (uint64_t)(i0 - 1));
        uint32_t rwB = load16(readA.arena, readB.pos + (uint64_t)(i0 - 1));  // one arena
        uint32_t rnA = readA.cnt ? nmask16(readA.iv, readA.cnt, i0 - 1) : 0u;
        uint32_t rnB = readB.cnt ? nmask16(readB.iv, readB.cnt, i0 - 1) : 0u;
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            uint32_t ca = (rwA >> (30 - 2 * r)) & 3u, cb = (rwB >> (30 - 2 * r)) & 3u;
            if ((rnA >> (31 - r)) & 1u) ca = 4;
            if ((rnB >> (31 - r)) & 1u) cb = 4;
            S.la[r] = s_lut[2 * ca];
            S.lb[r] = s_lut[2 * cb];
        }
        uint32_t diag = 0x00020002u;
        if (clo - 1 >= plo && clo - 1 <= phi) diag = rb[(size_t)(clo - 1 - plo) * 32].x;
        uint32_t *ta = tbA + (size_t)s * sw * 32, *tbq = tbB + (size_t)s * sw * 32;
        int a_end = min(lo7, chi);
        dp_cols2<1, true>(S, oe1, oe4, ex4, clo, a_end, diag, warena, wposA, wposB, rb, plo, phi, lo7, ta,
                          tbq);
        int b_beg = lo7 + 1, b_end = min(hi0 - 1, chi);
        if (b_beg <= b_end)
            dp_cols2<0, false>(S, oe1, oe4, ex4, b_beg, b_end, diag, warena, wposA, wposB, rb, plo, phi,
                               lo7, ta + (size_t)(b_beg - clo) * 32,
                               tbq + (size_t)(b_beg - clo) * 32);
        int c_beg = max(lo7 + 1, hi0);
        // the row windows again rather than kept live across the interior
#pragma unroll
        for (int r = 0; r < STRIP; r++)
            S.lohi[r] = (uint32_t)g.lo(i0 + r) | ((uint32_t)g.hi(i0 + r) << 16);
        if (c_beg <= chi)
            dp_cols2<1, true>(S, oe1, oe4, ex4, c_beg, chi, diag, warena, wposA, wposB, rb, plo, phi, lo7,
                              ta + (size_t)(c_beg - clo) * 32, tbq + (size_t)(c_beg - clo) * 32);
        // row bookkeeping in row order (extend.rs:795-827).  The best cell:
        // a strictly larger row maximum replaces it, both pairs at once with
        // the keep mask of the row maximum (row_max2)
#pragma unroll
        for (int r = 0; r < STRIP; r++) {
            if (r < nact) {
                const uint32_t keep = prmt(bestHp2 + 0x80008000u - S.rmax[r], 0u, 0xBB99u);
                bestHp2 = (bestHp2 & keep) | (S.rmax[r] & ~keep);
                bestI2 = (bestI2 & keep) | ((uint32_t)(i0 + r) * 0x10001u & ~keep);
                bestJ2 = (bestJ2 & keep) | (S.arg[r] & ~keep);
            }
        }
        // the first touching row, per pair, until both pairs have one.  A
        // touch needs a zero half in arg ^ lo (left edge) or, when hi < n, in
        // rmax ^ Hl (right edge); (x - 0x10001) & ~x has bit 15 of a half set
        // for every zero half (and may set it in the half above one), so a
        // strip whose rows have none for a pair still without a touch skips
        // the exact per-row tests
        uint32_t zero_halves = 0u;
        if (open_halves) {
#pragma unroll
            for (int r = 0; r < STRIP; r++) {
                if (r < nact) {
                    const uint32_t lo_r = (uint32_t)g.lo(i0 + r);
                    const uint32_t zl = S.arg[r] ^ (lo_r * 0x10001u);
                    zero_halves |= (zl - 0x00010001u) & ~zl;
                    if (g.hi(i0 + r) < n) {
                        const uint32_t zr = S.rmax[r] ^ S.Hl[r];
                        zero_halves |= (zr - 0x00010001u) & ~zr;
                    }
                }
            }
        }
        if (zero_halves & open_halves) {
#pragma unroll
            for (int r = 0; r < STRIP; r++) {
                if (r < nact) {
                    const int lo = g.lo(i0 + r), hi = g.hi(i0 + r);
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const uint32_t bit = 0x8000u << (16 * q);
                        if (open_halves & bit) {
                            const int argj = (int)((S.arg[r] >> (16 * q)) & 0xffffu);
                            const bool tr = (((S.rmax[r] ^ S.Hl[r]) >> (16 * q)) & 0xffffu) == 0;
                            if (argj == lo) {
                                trow2 |= (uint32_t)(i0 + r) << (16 * q);
                                tflags |= (1u | (lo <= 1 ? 2u : 0u)) << (2 * q);
                                open_halves &= ~bit;
                            } else if (hi < n && tr) {
                                trow2 |= (uint32_t)(i0 + r) << (16 * q);
                                tflags |= (hi >= n ? 2u : 0u) << (2 * q);
                                open_halves &= ~bit;
                            }
                        }
                    }
                }
            }
        }
        plo = lo7;
        phi = g.hi(i0 + STRIP - 1);
    }
    FA.bestHp = (int)(bestHp2 & 0xffffu);
    FA.best_i = (int)(bestI2 & 0xffffu);
    FA.best_j = (int)(bestJ2 & 0xffffu);
    FB.bestHp = (int)(bestHp2 >> 16);
    FB.best_i = (int)(bestI2 >> 16);
    FB.best_j = (int)(bestJ2 >> 16);
    FA.trow = (int)(trow2 & 0xffffu);
    FA.tleft = tflags & 1u;
    FA.tclamp = (tflags >> 1) & 1u;
    FB.trow = (int)(trow2 >> 16);
    FB.tleft = (tflags >> 2) & 1u;
    FB.tclamp = (tflags >> 3) & 1u;
}

// Out-of-line fill, finish and lone-pair paths of the paired kernel: one
// copy of each in the kernel's code, and their registers are not reserved
// across one another.
__device__ __noinline__ void fill2_call(const GotohConst &K, const uint32_t *__restrict__ s_lut,
                                        const PairSetup &A, const PairSetup &B, uint32_t *tbA,
                                        uint32_t *tbB, uint32_t *rb, FillResult &FA,
                                        FillResult &FB) {
    dp_fill2(K, s_lut, A.m, A.n, A.g, A.read, B.read, A.win.arena, A.win.pos, B.win.pos, tbA,
             tbB, A.sw, reinterpret_cast<uint2 *>(rb), FA, FB);
}

__device__ __noinline__ void finish_call(const GotohJob &job, const GotohConst &K,
                                         const int8_t *__restrict__ lut, uint32_t pi,
                                         PairSetup &S, const FillResult &F, const uint32_t *tb) {
    finish_pair<32>(job, K, lut, pi, S, F, tb);
}

// A pair without a partner of its geometry: the paired fill with itself in
// both lanes (the second lane's traceback lands in the slot's unused half),
// or, when its window has N (the paired fill takes N in reads only), the
// one-pair fill with its row buffer in that unused half (tb_words >=
// rb_words: a pair's traceback holds at least one strip of row-buffer width).
__device__ __noinline__ void lone_call(const GotohJob &job, const GotohConst &K,
                                       const uint32_t *__restrict__ s_lut,
                                       const int8_t *__restrict__ lut, uint32_t pi,
                                       PairSetup &S, uint32_t *tb, uint32_t *tbB, uint32_t *rb) {
    FillResult F, F2;
    if (S.win.cnt)
        F = dp_fill<true>(K, s_lut, S.m, S.n, S.g, S.read, S.win, tb, S.sw, tbB);
    else
        fill2_call(K, s_lut, S, S, tb, tbB, rb, F, F2);
    finish_pair<32>(job, K, lut, pi, S, F, tb);
}

// Work item (a, b): both pairs in one thread when their geometry matches and
// their windows carry no N; otherwise one after the other (b = NONE: a alone).
// The descriptors are resolved again after the fill rather than kept live
// across it.
constexpr uint32_t NO_PAIR = 0xffffffffu;

__device__ void process_item2(const GotohJob &job, const GotohConst &K,
                              const uint32_t *__restrict__ s_lut, const int8_t *__restrict__ lut,
                              uint32_t pa, uint32_t pb, uint32_t *tb, uint32_t *rb) {
    uint32_t *tbB = tb + job.tb_words * 32;  // second half of the thread's slot
    bool both;
    FillResult FA, FB;
    {
        PairSetup A, B;
        const bool ra = setup_pair(job, K, pa, job.tb_words, job.rb_words, true, A);
        const bool rb_ = pb != NO_PAIR && setup_pair(job, K, pb, job.tb_words, job.rb_words, true, B);
        both = ra && rb_ && A.m == B.m && A.n == B.n && A.full == B.full &&
               A.g.off == B.g.off && A.g.half == B.g.half && A.win.cnt == 0 && B.win.cnt == 0;
        if (both) {
            fill2_call(K, s_lut, A, B, tb, tbB, rb, FA, FB);
        } else {
            if (ra) lone_call(job, K, s_lut, lut, pa, A, tb, tbB, rb);
            if (rb_) lone_call(job, K, s_lut, lut, pb, B, tb, tbB, rb);
        }
    }
    if (both) {
        PairSetup A, B;
        setup_pair(job, K, pa, job.tb_words, job.rb_words, false, A);
        finish_call(job, K, lut, pa, A, FA, tb);
        setup_pair(job, K, pb, job.tb_words, job.rb_words, false, B);
        finish_call(job, K, lut, pb, B, FB, tbB);
    }
}

// Persistent paired kernel: work item k of the (class range of the) list is
// positions 2k and 2k + 1; neighbours in the binned list share their
// geometry key.  Scratch per warp: 2 x tb_words and 2 x rb_words words per
// lane.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) gotoh2_kernel(GotohJob job, GotohConst K) {
    __shared__ uint32_t s_lut[10];
    __shared__ int8_t s_lut25[32];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) s_lut[k] = K.lut4[k >> 1][k & 1];
#pragma unroll
        for (int k = 0; k < 25; k++) s_lut25[k] = K.lut[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t warp_slot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t *tb = job.tb + warp_slot * (2 * job.tb_words) * 32 + lane;
    uint32_t *rb = job.rb + warp_slot * (2 * job.rb_words) * 32 + 2 * lane;
    uint64_t b0 = 0, b1 = job.list_count ? (uint64_t)(*job.list_count) : job.n_pairs;
    if (job.range) {  // one length class of the binned list
        b0 = job.range[0];
        b1 = job.range[1] > job.range[0] ? job.range[1] : b0;
    }
    const uint64_t total = (b1 - b0 + 1) / 2;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd((unsigned long long *)job.queue, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        uint64_t k = base + lane;
        if (k < total) {
            uint64_t x = b0 + 2 * k, y = x + 1;
            uint32_t pa = job.list ? job.list[x] : (uint32_t)x;
            uint32_t pb = y < b1 ? (job.list ? job.list[y] : (uint32_t)y) : NO_PAIR;
            process_item2(job, K, s_lut, s_lut25, pa, pb, tb, rb);
        }
    }
}

int make_gotoh_const(const esp_extend_params &p, GotohConst &k) {
    // Device domain: substitution scores fit the 4*s int8 PRMT table and the
    // scaled gap keys fit int16 in the row buffer.  The reference's own
    // parameter sets (defaults 2/-4/4/2 and the 400/400 rescue pass) are inside.
    auto in8 = [](int v) { return v >= -32 && v <= 31; };
    if (!in8(p.match_score) || !in8(p.mismatch) || p.gap_open < 0 || p.gap_ext < 0 ||
        4LL * (p.gap_open + p.gap_ext) > 8000 || p.edit_dir < 0 || p.edit_dir > 2)
        return ESP_EDOMAIN;
    k.open_ext = -(p.gap_open + p.gap_ext);
    k.ext = -p.gap_ext;
    k.oe1 = 4 * k.open_ext - 1;
    k.oe4 = 4 * k.open_ext;
    k.ex4 = 4 * k.ext;
    k.match = p.match_score;
    k.edit_dir = p.edit_dir;
    // SubstLut (extend.rs:164-179): scores[read*5 + ref]
    int lut[25];
    for (int i = 0; i < 25; i++) lut[i] = (int16_t)p.mismatch;
    for (int c = 0; c < 4; c++) lut[c * 5 + c] = (int16_t)p.match_score;
    if (p.edit_dir == ESP_EDIT_AG) lut[10] = 0;  // read G / ref A
    if (p.edit_dir == ESP_EDIT_TC) lut[8] = 0;   // read C / ref T
    for (int i = 0; i < 25; i++) k.lut[i] = (int8_t)lut[i];
    // The row buffer keeps 4E (signed) and 4H + 2 in 16 bits, so every H and
    // E must stay <= 8191; H <= m * (largest substitution score).
    int smax = 0;
    for (int i = 0; i < 25; i++) smax = lut[i] > smax ? lut[i] : smax;
    k.max_m = smax > 0 ? 8191 / smax : 32767;
    // traceback kind of a diagonal step by read code * 5 + window code:
    // K_MM for equal ACGT codes, K_MZ for the edit-tolerated pair, K_MX
    // otherwise (a match and a tolerated pair exclude each other)
    k.dkind = 0;
    for (int q = 0; q < 5; q++)
        for (int c = 0; c < 5; c++) {
            const bool mz = (p.edit_dir == ESP_EDIT_AG && q == 2 && c == 0) ||
                            (p.edit_dir == ESP_EDIT_TC && q == 1 && c == 3);
            const int kd = (q == c && q < 4) ? K_MM : (mz ? K_MZ : K_MX);
            k.dkind |= (uint64_t)kd << (2 * (q * 5 + c));
        }
    for (int rc = 0; rc < 5; rc++) {
        uint32_t w[2] = {0, 0};
        for (int fc = 0; fc < 8; fc++) {
            int s = lut[rc * 5 + (fc < 4 ? fc : 4)];
            w[fc >> 2] |= (uint32_t)(uint8_t)(int8_t)(4 * s) << (8 * (fc & 3));
        }
        k.lut4[rc][0] = w[0];
        k.lut4[rc][1] = w[1];
    }
    return ESP_OK;
}

void gotoh_scratch_words(uint32_t m, uint32_t n, int32_t half, uint64_t &tb, uint64_t &rb) {
    bool full = half < 0;
    int64_t h = full ? n : half;
    int64_t sw = full ? n : (2 * h + STRIP < (int64_t)n ? 2 * h + STRIP : (int64_t)n);
    tb = (uint64_t)((m + STRIP - 1) / STRIP) * (uint64_t)sw;
    rb = (uint64_t)sw;
}

// Kernel variants: 0, 1 = one pair per thread at 3 / 4 resident blocks per
// SM; 2, 3 = two pairs per thread (16x2 lanes) at 3 / 4.  More blocks mean
// fewer registers per thread (spills) but more warps to hide latency; which
// wins depends on the band width, so the host picks per length class (the
// tuning in abi.cu).
int gotoh_blocks_per_sm(int block, int variant) {
    int nb = 0;
    cudaError_t e;
    switch (variant) {
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gotoh_kernel<3>, block, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gotoh2_kernel<3>, block, 0); break;
    case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gotoh2_kernel<4>, block, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gotoh_kernel<4>, block, 0);
    }
    if (e != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

cudaError_t launch_gotoh(const GotohJob &job, const GotohConst &k, int warps, int block,
                         cudaStream_t st, int variant) {
    int threads = warps * 32;
    int grid = (threads + block - 1) / block;
    switch (variant) {
    case 0: gotoh_kernel<3><<<grid, block, 0, st>>>(job, k); break;
    case 2: gotoh2_kernel<3><<<grid, block, 0, st>>>(job, k); break;
    case 3: gotoh2_kernel<4><<<grid, block, 0, st>>>(job, k); break;
    default: gotoh_kernel<4><<<grid, block, 0, st>>>(job, k);
    }
    return cudaGetLastError();
}

}  // namespace esp
