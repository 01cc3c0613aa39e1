/*
 * myers.c -- oracle restatement of the two EA-Myers formulations:
 *   crates/map/src/myers_ea.rs     (edlib-form block carry, u128 blocks)
 *   crates/engine/src/myers.rs     (ripple-carry block chain, u128 blocks)
 * plus an independent O(m*n) DP used to pin both.  TEST INFRASTRUCTURE ONLY.
 */
#include "esp_oracle.h"

#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
#define U128_MAX (~(u128)0)
#define LONG_MAX_M 256

static uint8_t upper(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }

/* myers_ea.rs:18-24 mask_for */
static u128 mask_for(int64_t m) { return m >= 128 ? U128_MAX : (((u128)1 << m) - 1); }

/* myers_ea.rs:28-38 ea_matches */
static int ea_matches(uint8_t read, uint8_t ref) {
    uint8_t r = upper(read), f = upper(ref);
    switch (r) {
    case 'A': return f == 'A';
    case 'C': return f == 'C' || f == 'T';
    case 'G': return f == 'G' || f == 'A';
    case 'T': return f == 'T';
    default: return 0;
    }
}

/* myers_ea.rs:42-56 build_peq; :195-217 build_peq_2block (blk selects the
 * 128-position block). */
static void build_peq_blk(const uint8_t *read, int64_t m, int blk, u128 peq[256]) {
    memset(peq, 0, 256 * sizeof(u128));
    static const uint8_t ACGT[4] = {'A', 'C', 'G', 'T'};
    int64_t lo = (int64_t)blk * 128, hi = lo + 128 < m ? lo + 128 : m;
    for (int64_t i = lo; i < hi; i++)
        for (int f = 0; f < 4; f++)
            if (ea_matches(read[i], ACGT[f])) peq[ACGT[f]] |= (u128)1 << (i - lo);
    peq['a'] = peq['A'];
    peq['c'] = peq['C'];
    peq['g'] = peq['G'];
    peq['t'] = peq['T'];
}

/* myers_ea.rs:64-91 calculate_block (edlib form) */
static void calc_block_ea(u128 pv, u128 mv, u128 eq_in, int hin, u128 mask, u128 high_bit,
                          u128 *pv_out, u128 *mv_out, int *hout) {
    u128 hin_is_neg = (u128)(hin < 0);
    u128 ph_bit0 = (u128)(hin > 0);
    u128 xv = eq_in | mv;
    u128 eq = eq_in | hin_is_neg;
    u128 xh = (((eq & pv) + pv) ^ pv) | eq;
    u128 ph = mv | ~(xh | pv);
    u128 mh = pv & xh;
    *hout = (ph & high_bit) ? 1 : ((mh & high_bit) ? -1 : 0);
    u128 ph_sh = (ph << 1) | ph_bit0;
    u128 mh_sh = (mh << 1) | hin_is_neg;
    *pv_out = (mh_sh | ~(xv | ph_sh)) & mask;
    *mv_out = (ph_sh & xv) & mask;
}

/* myers_ea.rs:93-116 scan (single block) with the best-end update of
 * :147-151 (strict <, earliest end wins). */
static void scan1(const u128 peq[256], int64_t m, const uint8_t *text, int64_t n,
                  int32_t *best_out, int64_t *at_out) {
    u128 mask = mask_for(m);
    u128 high = (u128)1 << (m - 1);
    u128 vp = mask, vn = 0;
    int32_t score = (int32_t)m, best = score;
    int64_t best_at = 0;
    for (int64_t j = 0; j < n; j++) {
        u128 nvp, nvn;
        int hout;
        calc_block_ea(vp, vn, peq[text[j]], 0, mask, high, &nvp, &nvn, &hout);
        vp = nvp;
        vn = nvn;
        score += hout;
        if (score < best) {
            best = score;
            best_at = j + 1;
        }
    }
    *best_out = best;
    *at_out = best_at;
}

/* myers_ea.rs:219-247 scan2 (two chained blocks, block 1 takes hin = hout0) */
static void scan2(const u128 peq0[256], const u128 peq1[256], int64_t m, const uint8_t *text,
                  int64_t n, int32_t *best_out, int64_t *at_out) {
    int64_t m1 = m - 128;
    u128 mask1 = mask_for(m1);
    u128 high0 = (u128)1 << 127, high1 = (u128)1 << (m1 - 1);
    u128 vp0 = U128_MAX, vn0 = 0, vp1 = mask1, vn1 = 0;
    int32_t score = (int32_t)m, best = score;
    int64_t best_at = 0;
    for (int64_t j = 0; j < n; j++) {
        u128 a, b, c, d;
        int h0, h1;
        calc_block_ea(vp0, vn0, peq0[text[j]], 0, U128_MAX, high0, &a, &b, &h0);
        calc_block_ea(vp1, vn1, peq1[text[j]], h0, mask1, high1, &c, &d, &h1);
        vp0 = a; vn0 = b; vp1 = c; vn1 = d;
        score += h1;
        if (score < best) {
            best = score;
            best_at = j + 1;
        }
    }
    *best_out = best;
    *at_out = best_at;
}

/* Single-block entry points (myers_ea.rs:118-185).  For 128 < m <= 256 the
 * reference computes `1u128 << (m - 1)`, a shift overflow (a panic in debug
 * builds); its callers route those lengths to long::* (align.rs:878-882,
 * :1791-1799), so the oracle rejects them. */
static int single_best_end(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                           int32_t *dist, int64_t *end) {
    if (m == 0) { *dist = 0; *end = 0; return ORC_OK; }
    if (m > LONG_MAX_M) { *dist = (int32_t)m; *end = 0; return ORC_OK; }
    if (m > 128) return ORC_EINVAL;
    u128 *peq = (u128 *)malloc(256 * sizeof(u128));
    if (!peq) return ORC_ENOMEM;
    build_peq_blk(read, m, 0, peq);
    scan1(peq, m, text, n, dist, end);
    free(peq);
    return ORC_OK;
}

int orc_myers_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                    int32_t *dist) {
    int64_t e;
    return single_best_end(read, m, text, n, dist, &e);
}

int orc_myers_infix_best_end(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                             int32_t *dist, int64_t *end) {
    return single_best_end(read, m, text, n, dist, end);
}

static int reversed_call(int (*fn)(const uint8_t *, int64_t, const uint8_t *, int64_t,
                                   int32_t *, int64_t *),
                         const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                         int32_t *dist, int64_t *start) {
    if (m == 0) { *dist = 0; *start = 0; return ORC_OK; }
    if (m > LONG_MAX_M) { *dist = (int32_t)m; *start = 0; return ORC_OK; }
    uint8_t *rr = (uint8_t *)malloc((size_t)(m + n + 1));
    if (!rr) return ORC_ENOMEM;
    uint8_t *rt = rr + m;
    for (int64_t k = 0; k < m; k++) rr[k] = read[m - 1 - k];
    for (int64_t k = 0; k < n; k++) rt[k] = text[n - 1 - k];
    int64_t rev_end = 0;
    int rc = fn(rr, m, rt, n, dist, &rev_end);
    free(rr);
    if (rc == ORC_OK) *start = n - rev_end;
    return rc;
}

int orc_myers_infix_best_start(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                               int32_t *dist, int64_t *start) {
    return reversed_call(single_best_end, read, m, text, n, dist, start);
}

/* long::* (myers_ea.rs:249-310): m <= 128 dispatches to the single block. */
int orc_myers_long_infix_best_end(const uint8_t *read, int64_t m, const uint8_t *text,
                                  int64_t n, int32_t *dist, int64_t *end) {
    if (m <= 128) return single_best_end(read, m, text, n, dist, end);
    if (m > LONG_MAX_M) { *dist = (int32_t)m; *end = 0; return ORC_OK; }
    u128 *peq = (u128 *)malloc(512 * sizeof(u128));
    if (!peq) return ORC_ENOMEM;
    build_peq_blk(read, m, 0, peq);
    build_peq_blk(read, m, 1, peq + 256);
    scan2(peq, peq + 256, m, text, n, dist, end);
    free(peq);
    return ORC_OK;
}

int orc_myers_long_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                         int32_t *dist) {
    int64_t e;
    return orc_myers_long_infix_best_end(read, m, text, n, dist, &e);
}

int orc_myers_long_infix_best_start(const uint8_t *read, int64_t m, const uint8_t *text,
                                    int64_t n, int32_t *dist, int64_t *start) {
    return reversed_call(orc_myers_long_infix_best_end, read, m, text, n, dist, start);
}

/* ---- crates/engine/src/myers.rs ---- */

/* :18-27 code5 */
static int code5(uint8_t b) {
    switch (b) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

typedef struct {
    int64_t m;
    int blocks;
    u128 peq[2][5];
    u128 init_pv[2];
    u128 top[2];
} myers_ea_t;

/* :76-106 MyersEa::new (asserts 1 <= m <= 256) */
static int engine_new(const uint8_t *pat, int64_t m, myers_ea_t *s) {
    if (m < 1 || m > 256) return ORC_EINVAL;
    memset(s, 0, sizeof(*s));
    s->m = m;
    s->blocks = (int)((m + 127) / 128);
    for (int64_t i = 0; i < m; i++) s->peq[i / 128][code5(pat[i])] |= (u128)1 << (i % 128);
    int64_t b0 = m < 128 ? m : 128;
    s->init_pv[0] = b0 == 128 ? U128_MAX : (((u128)1 << b0) - 1);
    s->top[0] = (u128)1 << (b0 - 1);
    if (s->blocks == 2) {
        int64_t b1 = m - 128;
        s->init_pv[1] = b1 == 128 ? U128_MAX : (((u128)1 << b1) - 1);
        s->top[1] = (u128)1 << (b1 - 1);
    }
    return ORC_OK;
}

/* :111-123 eq_vec */
static u128 eq_vec(const myers_ea_t *s, int blk, int tcode) {
    if (tcode > 3) return 0;
    u128 eq = s->peq[blk][tcode];
    if (tcode == 0) eq |= s->peq[blk][2];
    else if (tcode == 3) eq |= s->peq[blk][1];
    return eq;
}

/* :179-208 calculate_block with explicit adder carry */
static int engine_block(u128 eq, u128 *pv, u128 *mv, int hin, int cin, u128 top, int *cout) {
    u128 xv = eq | *mv;
    u128 a = eq & *pv;
    u128 sum = a + *pv;
    int c1 = sum < a;
    u128 sum2 = sum + (u128)(cin ? 1 : 0);
    int c2 = sum2 < sum;
    *cout = c1 | c2;
    u128 xh = (sum2 ^ *pv) | xv;
    u128 ph = *mv | ~(xh | *pv);
    u128 mh = *pv & xh;
    int hout = 0;
    if (ph & top) hout = 1;
    else if (mh & top) hout = -1;
    ph <<= 1;
    mh <<= 1;
    if (hin == 1) ph |= 1;
    else if (hin == -1) mh |= 1;
    *pv = mh | ~(xv | ph);
    *mv = ph & xv;
    return hout;
}

static uint32_t engine_run(const myers_ea_t *s, const uint8_t *text, int64_t n, int global) {
    u128 pv[2] = {s->init_pv[0], s->init_pv[1]}, mv[2] = {0, 0};
    int32_t score = (int32_t)s->m;
    uint32_t best = (uint32_t)s->m;
    for (int64_t j = 0; j < n; j++) {
        int tcode = code5(text[j]);
        int hin = global ? 1 : 0, cin = 0;
        for (int blk = 0; blk < s->blocks; blk++) {
            int cout;
            int h = engine_block(eq_vec(s, blk, tcode), &pv[blk], &mv[blk], hin, cin,
                                 s->top[blk], &cout);
            hin = h;
            cin = cout;
        }
        score += hin;
        if (!global && score >= 0 && (uint32_t)score < best) best = (uint32_t)score;
    }
    if (global) return (uint32_t)(score > 0 ? score : 0);
    return best;
}

/* :32-38 infix / :52-56 long::infix (same matcher; the single-block entry's
 * m <= 128 is a debug assertion only, the matcher covers 256). */
int orc_engine_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                     uint32_t *dist) {
    myers_ea_t s;
    int rc = engine_new(read, m, &s);
    if (rc != ORC_OK) return rc;
    *dist = engine_run(&s, text, n, 0);
    return ORC_OK;
}

/* :42-44 global / :58-62 long::global */
int orc_engine_global(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                      uint32_t *dist) {
    myers_ea_t s;
    int rc = engine_new(read, m, &s);
    if (rc != ORC_OK) return rc;
    *dist = engine_run(&s, text, n, 1);
    return ORC_OK;
}

/* Independent semi-global EA edit distance: D[0][j] = 0, D[i][0] = i,
 * substitution free when ea_matches(read[i-1], text[j-1]).  Reports the
 * minimum over j >= 0 of D[m][j] (j = 0 included, so an empty text gives m)
 * and the earliest j attaining it (0 when D[m][0] = m is never beaten). */
int orc_ea_edit_dp(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                   int32_t *dist, int64_t *end) {
    int32_t *col = (int32_t *)malloc((size_t)(m + 1) * sizeof(int32_t));
    if (!col) return ORC_ENOMEM;
    for (int64_t i = 0; i <= m; i++) col[i] = (int32_t)i;
    int32_t best = (int32_t)m;
    int64_t best_at = 0;
    for (int64_t j = 1; j <= n; j++) {
        int32_t diag = col[0];
        col[0] = 0;
        for (int64_t i = 1; i <= m; i++) {
            int32_t up = col[i];
            int32_t v = diag + (ea_matches(read[i - 1], text[j - 1]) ? 0 : 1);
            if (up + 1 < v) v = up + 1;
            if (col[i - 1] + 1 < v) v = col[i - 1] + 1;
            diag = up;
            col[i] = v;
        }
        if (col[m] < best) {
            best = col[m];
            best_at = j;
        }
    }
    free(col);
    *dist = best;
    *end = best_at;
    return ORC_OK;
}
