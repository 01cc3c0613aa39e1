/*
 * extend.c -- oracle restatement of crates/map/src/extend.rs (scalar kernel,
 * traceback/end trimming/neutral flanks, dispatch and the two-attempt
 * extend_hint policy).  TEST INFRASTRUCTURE ONLY (see esp_oracle.h).
 *
 * The reference's AVX2 kernels (extend.rs:1095-2026) are documented and
 * tested as cell-for-cell identical to run_band::<i16>; the oracle therefore
 * restates the scalar kernel, which is also what the reference executes on
 * an aarch64 host (the AVX2 dispatch is cfg(target_arch = "x86_64")).
 */
#include "esp_oracle.h"

#include <stdlib.h>
#include <string.h>

/* DP cells computed by run_band on this thread (rows 1..m window widths);
 * read by the batch drivers for the CPU-baseline cell census. */
_Thread_local int64_t orc_tls_cells = 0;

/* extend.rs:601-604 */
enum { H_DIAG = 0, H_FROM_E = 1, H_FROM_F = 2, H_START = 3 };

/* extend.rs:126 */
#define INITIAL_BAND 30

/* extend.rs:150-159 base_code */
int orc_base_code(uint8_t b) {
    switch (b) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

/* extend.rs:87-93 exempt_dir: 1 = plus (ref A / read G), 0 = minus
 * (ref T / read C), -1 = not an editing pair. */
static int exempt_dir(uint8_t ref_b, uint8_t read_b) {
    if (ref_b == 'A' && read_b == 'G') return 1;
    if (ref_b == 'T' && read_b == 'C') return 0;
    return -1;
}

/* extend.rs:71-76 EditDir::exempt */
static int edit_exempt(int dir, uint8_t ref_b, uint8_t read_b) {
    int e = exempt_dir(ref_b, read_b);
    return (dir == ORC_EDIT_AG && e == 1) || (dir == ORC_EDIT_TC && e == 0);
}

/* extend.rs:164-179 SubstLut::new (scores[read*5 + ref]) */
void orc_lut(const orc_params *p, int16_t lut[25]) {
    int16_t m = (int16_t)p->match_score, mm = (int16_t)p->mismatch;
    for (int k = 0; k < 25; k++) lut[k] = mm;
    for (int c = 0; c < 4; c++) lut[c * 5 + c] = m;
    if (edit_exempt(p->edit_dir, 'A', 'G')) lut[10] = 0;
    if (edit_exempt(p->edit_dir, 'T', 'C')) lut[8] = 0;
}

/* extend.rs:444-460 CoreParams */
typedef struct {
    int16_t lut[25];
    int32_t open_ext;
    int32_t ext;
} core_params;

static void core_new(const orc_params *p, core_params *c) {
    orc_lut(p, c->lut);
    c->open_ext = -(p->gap_open + p->gap_ext);
    c->ext = -p->gap_ext;
}

/* extend.rs:471-528 Acc for i16 / i32.  Values are held in int32 for both;
 * the i16 flavour reproduces the 16-bit wrap of release-mode arithmetic and
 * the max(NEG) clamp. */
#define NEG16 (-30000)
#define NEG32 (-1000000000)

int16_t orc_i16_add(int16_t a, int16_t b) {
    if (a == NEG16 || b == NEG16) return NEG16;
    int16_t s = (int16_t)(uint16_t)((uint16_t)a + (uint16_t)b);
    return s > NEG16 ? s : NEG16;
}

static inline int32_t acc_add(int wide, int32_t a, int32_t b) {
    if (wide) {
        if (a == NEG32 || b == NEG32) return NEG32;
        return (int32_t)((uint32_t)a + (uint32_t)b);
    }
    return orc_i16_add((int16_t)a, (int16_t)b);
}

static inline int32_t acc_from(int wide, int32_t v) {
    return wide ? v : (int32_t)(int16_t)(uint16_t)v;
}

/* ---- CIGAR helpers ---- */
typedef struct {
    uint32_t *v;
    uint32_t n, cap;
} opvec;

static int opvec_push_raw(opvec *o, uint32_t op) {
    if (o->n == o->cap) {
        uint32_t nc = o->cap ? o->cap * 2 : 16;
        uint32_t *nv = (uint32_t *)realloc(o->v, nc * sizeof(uint32_t));
        if (!nv) return ORC_ENOMEM;
        o->v = nv;
        o->cap = nc;
    }
    o->v[o->n++] = op;
    return ORC_OK;
}

/* extend.rs:254-282 push_op: merge with the previous op of the same kind. */
static int push_op(opvec *o, uint32_t code, uint32_t len) {
    if (o->n > 0 && (o->v[o->n - 1] & 15u) == code) {
        o->v[o->n - 1] += len << 4;
        return ORC_OK;
    }
    return opvec_push_raw(o, (len << 4) | code);
}

static int emit(orc_ext *out, const opvec *ops) {
    out->n_ops = ops->n;
    if (out->ops && out->cap) {
        uint32_t k = ops->n < out->cap ? ops->n : out->cap;
        memcpy(out->ops, ops->v, k * sizeof(uint32_t));
    }
    return (ops->n > out->cap) ? ORC_ECAP : ORC_OK;
}

/* extend.rs:430-442 empty_extension */
static int empty_extension(uint32_t read_len, orc_ext *out) {
    out->read_start = out->read_end = out->ref_start = 0;
    out->score = 0;
    out->n_ops = read_len > 0 ? 1 : 0;
    if (read_len > 0) {
        if (out->cap < 1 || !out->ops) return ORC_ECAP;
        out->ops[0] = (read_len << 4) | ORC_OP_S;
    }
    return ORC_OK;
}

typedef struct {
    int64_t lo;
    size_t off, len;
} row_trace;

typedef struct {
    uint8_t op;
    int32_t d;
} step_t;

/* extend.rs:864-1068 finish_extension: state-machine traceback, end
 * trimming, coordinate/CIGAR rebuild and neutral flank extension. */
static int finish_extension(int64_t m, const core_params *core, const row_trace *rows,
                            const uint8_t *rows_flat, const uint8_t *read_codes,
                            const uint8_t *ref_codes, int64_t n_ref, int64_t best_i,
                            int64_t best_j, orc_ext *out) {
    size_t cap_steps = (size_t)(m + n_ref + 4);
    step_t *steps = (step_t *)malloc(cap_steps * sizeof(step_t));
    if (!steps) return ORC_ENOMEM;
    size_t n_steps = 0;
    enum { TB_H, TB_E, TB_F } state = TB_H;
    int64_t i = best_i, j = best_j;
    for (;;) {
        if (i <= 0 || j <= 0) break;
        const row_trace *row = &rows[i];
        if (j < row->lo || j >= row->lo + (int64_t)row->len) break;
        uint8_t cell = rows_flat[row->off + (size_t)(j - row->lo)];
        if (state == TB_H) {
            int h = cell & 3;
            if (h == H_DIAG) {
                int32_t s = core->lut[read_codes[i - 1] * 5 + ref_codes[j - 1]];
                steps[n_steps++] = (step_t){ORC_OP_M, s};
                i -= 1;
                j -= 1;
            } else if (h == H_FROM_E) {
                steps[n_steps++] = (step_t){ORC_OP_I, core->open_ext};
                state = ((cell >> 2) & 1) ? TB_E : TB_H;
                i -= 1;
            } else if (h == H_FROM_F) {
                steps[n_steps++] = (step_t){ORC_OP_D, core->open_ext};
                state = ((cell >> 4) & 1) ? TB_F : TB_H;
                j -= 1;
            } else {
                break; /* H_START */
            }
        } else if (state == TB_E) {
            steps[n_steps++] = (step_t){ORC_OP_I, core->ext};
            if (((cell >> 2) & 1) == 0) state = TB_H;
            i -= 1;
        } else {
            steps[n_steps++] = (step_t){ORC_OP_D, core->ext};
            if (((cell >> 4) & 1) == 0) state = TB_H;
            j -= 1;
        }
    }
    /* steps.reverse() */
    for (size_t a = 0, b = n_steps ? n_steps - 1 : 0; a < b; a++, b--) {
        step_t t = steps[a];
        steps[a] = steps[b];
        steps[b] = t;
    }

    size_t lead = 0, trail = 0;
    {
        int32_t acc = 0;
        for (size_t k = 0; k < n_steps; k++) {
            acc += steps[k].d;
            if (acc <= 0) lead = k + 1;
        }
    }
    {
        int32_t acc = 0;
        for (size_t kk = n_steps; kk-- > 0;) {
            acc += steps[kk].d;
            if (acc <= 0) trail = n_steps - kk;
        }
    }
    if (n_steps > 0 && lead + trail >= n_steps) {
        lead = n_steps / 2;
        trail = n_steps - lead - 1;
    }
    uint32_t read_start = (uint32_t)(i > 0 ? i : 0);
    uint32_t ref_start = (uint32_t)(j > 0 ? j : 0);
    for (size_t k = 0; k < lead; k++) {
        if (steps[k].op == ORC_OP_M || steps[k].op == ORC_OP_I) read_start++;
        if (steps[k].op == ORC_OP_M || steps[k].op == ORC_OP_D) ref_start++;
    }

    int32_t score = 0;
    opvec ops = {0};
    uint32_t rm = 0, used_ref = 0;
    int rc = ORC_OK;
    for (size_t k = lead; k < n_steps - trail; k++) {
        score += steps[k].d;
        if ((rc = push_op(&ops, steps[k].op, 1)) != ORC_OK) goto done;
        if (steps[k].op == ORC_OP_M || steps[k].op == ORC_OP_I) rm++;
        if (steps[k].op == ORC_OP_M || steps[k].op == ORC_OP_D) used_ref++;
    }
    uint32_t read_end = read_start + rm;
    if (score > 0) {
        /* neutral_column (:998-1000): both ACGT and equal or an editing pair */
        static const uint8_t ACGT[4] = {'A', 'C', 'G', 'T'};
        uint32_t neutral_left = 0;
        int32_t delta = 0;
        uint32_t lim = read_start < ref_start ? read_start : ref_start;
        for (uint32_t nn = 1; nn <= lim; nn++) {
            int q = read_codes[read_start - nn], r = ref_codes[ref_start - nn];
            if (!(q < 4 && r < 4 && (q == r || exempt_dir(ACGT[r], ACGT[q]) >= 0))) break;
            delta += core->lut[q * 5 + r];
            if (delta == 0) neutral_left = nn;
        }
        uint32_t ref_end = ref_start + used_ref;
        uint32_t neutral_right = 0;
        delta = 0;
        uint32_t av1 = (uint32_t)m - read_end, av2 = (uint32_t)n_ref - ref_end;
        uint32_t available = av1 < av2 ? av1 : av2;
        for (uint32_t nn = 0; nn < available; nn++) {
            int q = read_codes[read_end + nn], r = ref_codes[ref_end + nn];
            if (!(q < 4 && r < 4 && (q == r || exempt_dir(ACGT[r], ACGT[q]) >= 0))) break;
            delta += core->lut[q * 5 + r];
            if (delta == 0) neutral_right = nn + 1;
        }
        if (neutral_left > 0 || neutral_right > 0) {
            opvec ex = {0};
            if (neutral_left > 0 && (rc = push_op(&ex, ORC_OP_M, neutral_left)) != ORC_OK) {
                free(ex.v);
                goto done;
            }
            for (uint32_t k = 0; k < ops.n; k++)
                if ((rc = push_op(&ex, ops.v[k] & 15u, ops.v[k] >> 4)) != ORC_OK) {
                    free(ex.v);
                    goto done;
                }
            if (neutral_right > 0 && (rc = push_op(&ex, ORC_OP_M, neutral_right)) != ORC_OK) {
                free(ex.v);
                goto done;
            }
            free(ops.v);
            ops = ex;
            read_start -= neutral_left;
            ref_start -= neutral_left;
            read_end += neutral_right;
        }
    }
    {
        opvec cig = {0};
        if (read_start > 0) rc = push_op(&cig, ORC_OP_S, read_start);
        for (uint32_t k = 0; rc == ORC_OK && k < ops.n; k++)
            rc = push_op(&cig, ops.v[k] & 15u, ops.v[k] >> 4);
        if (rc == ORC_OK && read_end < (uint32_t)m)
            rc = push_op(&cig, ORC_OP_S, (uint32_t)m - read_end);
        if (rc == ORC_OK) {
            out->read_start = read_start;
            out->read_end = read_end;
            out->ref_start = ref_start;
            out->score = score;
            rc = emit(out, &cig);
        }
        free(cig.v);
    }
done:
    free(ops.v);
    free(steps);
    return rc;
}

/* extend.rs:606-851 run_band<T>.  `wide` picks the accumulator (i16 with
 * sentinel clamp, or i32). */
int orc_run_band(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                 const orc_params *p, int wide, int has_band, int64_t offset, int64_t num,
                 int64_t den, int64_t half, orc_ext *out, orc_touch *touch) {
    memset(touch, 0, sizeof(*touch));
    if (m == 0 || n == 0) return empty_extension((uint32_t)m, out);
    core_params core;
    core_new(p, &core);
    if (has_band) {
        den = den > 1 ? den : 1;
        half = half > 0 ? half : 0;
    } else {
        offset = 0;
        num = 1;
        den = 1;
        half = n;
    }
    /* The reference asserts num == den == 1 (debug_assert at :633); every
     * call site passes 1/1. */
    if (num != 1 || den != 1) return ORC_EINVAL;
    const int32_t NEG = wide ? NEG32 : NEG16;
    int64_t width = 2 * half + 1;
    int32_t *buf = (int32_t *)malloc((size_t)width * 5 * sizeof(int32_t));
    uint8_t *rc8 = (uint8_t *)malloc((size_t)(m + n));
    row_trace *rows = (row_trace *)malloc((size_t)(m + 1) * sizeof(row_trace));
    int64_t rowcap = width < n + 1 ? width : n + 1;
    uint8_t *flat = (uint8_t *)malloc((size_t)((m + 1) * rowcap + 1));
    if (!buf || !rc8 || !rows || !flat) {
        free(buf); free(rc8); free(rows); free(flat);
        return ORC_ENOMEM;
    }
    int32_t *h_prev = buf, *h_cur = buf + width, *e_prev = buf + 2 * width,
            *e_cur = buf + 3 * width, *f_cur = buf + 4 * width;
    for (int64_t k = 0; k < width * 5; k++) buf[k] = NEG;
    uint8_t *read_codes = rc8, *ref_codes = rc8 + m;
    for (int64_t k = 0; k < m; k++) read_codes[k] = (uint8_t)orc_base_code(read[k]);
    for (int64_t k = 0; k < n; k++) ref_codes[k] = (uint8_t)orc_base_code(rf[k]);
    size_t flat_len = 0;

    int64_t center0 = offset;
    int64_t lo0 = center0 - half > 0 ? center0 - half : 0;
    int64_t hi0 = center0 + half < n ? center0 + half : n;
    if (lo0 <= hi0) {
        size_t len = (size_t)(hi0 - lo0 + 1);
        memset(flat, H_START, len);
        for (size_t c = 0; c < len; c++) h_prev[c] = acc_from(wide, 0);
        rows[0] = (row_trace){lo0, 0, len};
        flat_len = len;
    } else {
        rows[0] = (row_trace){lo0, 0, 0};
    }
    const int32_t open_ext = acc_from(wide, core.open_ext);
    const int32_t ext_p = acc_from(wide, core.ext);
    const int32_t zero = 0;
    int32_t best_score = zero;
    int64_t best_i = 0, best_j = 0;
    int64_t plo = lo0, phi = hi0;
    for (int64_t i = 1; i <= m; i++) {
        int64_t center = offset + i;
        int64_t c = center < 1 ? 1 : (center > n ? n : center);
        int64_t lo = c - half > 1 ? c - half : 1;
        int64_t hi = c + half < n ? c + half : n;
        if (lo > hi) {
            rows[i] = (row_trace){lo, flat_len, 0};
            plo = lo;
            phi = hi;
            continue;
        }
        size_t off = flat_len;
        size_t len = (size_t)(hi - lo + 1);
        flat_len += len;
        int rc = read_codes[i - 1];
        int32_t row_max = NEG;
        int64_t row_max_cell = 0;
        for (int64_t jj = lo; jj <= hi; jj++) {
            size_t cidx = (size_t)(jj - lo);
            int in_prev = jj >= plo && jj <= phi;
            int32_t h_up = in_prev ? h_prev[jj - plo] : zero;
            int32_t e_up = in_prev ? e_prev[jj - plo] : NEG;
            int32_t e_open = acc_add(wide, h_up, open_ext);
            int32_t e_ext = acc_add(wide, e_up, ext_p);
            int32_t e_val;
            uint8_t edir;
            if (e_ext > e_open) { e_val = e_ext; edir = 1; } else { e_val = e_open; edir = 0; }

            int32_t h_left = jj > lo ? h_cur[cidx - 1] : zero;
            int32_t f_left = jj > lo ? f_cur[cidx - 1] : NEG;
            int32_t f_open = acc_add(wide, h_left, open_ext);
            int32_t f_ext = acc_add(wide, f_left, ext_p);
            int32_t f_val;
            uint8_t fdir;
            if (f_ext > f_open) { f_val = f_ext; fdir = 1; } else { f_val = f_open; fdir = 0; }

            int64_t hpi = jj - 1;
            int32_t h_diag = (hpi >= plo && hpi <= phi) ? h_prev[hpi - plo] : zero;
            int32_t s = core.lut[rc * 5 + ref_codes[jj - 1]];
            int32_t diag = acc_add(wide, h_diag, acc_from(wide, s));

            int32_t h_val = zero;
            uint8_t hdir = H_START;
            if (f_val != NEG && !(h_val > f_val)) { h_val = f_val; hdir = H_FROM_F; }
            if (e_val != NEG && !(h_val > e_val)) { h_val = e_val; hdir = H_FROM_E; }
            if (diag != NEG && !(h_val > diag)) { h_val = diag; hdir = H_DIAG; }
            if (h_val == zero) hdir = H_START;

            h_cur[cidx] = h_val;
            e_cur[cidx] = e_val;
            f_cur[cidx] = f_val;
            flat[off + cidx] = (uint8_t)(hdir | (edir << 2) | (fdir << 4));
            if (h_val > row_max) {
                row_max = h_val;
                row_max_cell = (int64_t)cidx;
            }
        }
        int left_strict = lo > 0;
        int right_strict = hi < n;
        if (!touch->touched) {
            if (left_strict && h_cur[0] == row_max) {
                *touch = (orc_touch){1, i, 1, lo <= 1};
            } else if (right_strict && h_cur[len - 1] == row_max) {
                *touch = (orc_touch){1, i, 0, hi >= n};
            }
        }
        if (row_max > best_score) {
            best_score = row_max;
            best_i = i;
            best_j = lo + row_max_cell;
        }
        rows[i] = (row_trace){lo, off, len};
        int32_t *t;
        t = h_prev; h_prev = h_cur; h_cur = t;
        t = e_prev; e_prev = e_cur; e_cur = t;
        plo = lo;
        phi = hi;
    }
    orc_tls_cells += (int64_t)(flat_len - rows[0].len);
    int rcode = finish_extension(m, &core, rows, flat, read_codes, ref_codes, n, best_i,
                                 best_j, out);
    free(buf);
    free(rc8);
    free(rows);
    free(flat);
    return rcode;
}

/* extend.rs:284-287 pure_byte */
static int pure_byte(uint8_t b) {
    return b == 'A' || b == 'C' || b == 'G' || b == 'T' || b == 'N';
}

/* extend.rs:293-344 run_dispatch (the AVX2 branches are cell-identical to
 * the i16 scalar kernel, so the pure path runs it directly). */
int orc_run_dispatch(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                     const orc_params *p, int has_band, int64_t offset, int64_t num,
                     int64_t den, int64_t half, orc_ext *out, orc_touch *touch) {
    int pure = 1;
    for (int64_t k = 0; k < m && pure; k++) pure = pure_byte(read[k]);
    for (int64_t k = 0; k < n && pure; k++) pure = pure_byte(rf[k]);
    return orc_run_band(read, m, rf, n, p, pure ? 0 : 1, has_band, offset, num, den, half,
                        out, touch);
}

int orc_extend(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
               const orc_params *p, orc_ext *out) {
    orc_touch t;
    return orc_run_dispatch(read, m, rf, n, p, 0, 0, 1, 1, 0, out, &t);
}

/* extend.rs:392-428 extend_hint; with force_i32 every attempt runs the i32
 * flavour of run_band (extend.rs:462-528) instead of run_dispatch's choice,
 * which is what the wide device kernel reproduces for reads whose scores
 * leave the i16 range. */
static int extend_hint_impl(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                            const orc_params *p, int64_t offset, uint32_t num, uint32_t den,
                            orc_ext *out, int *escalated, int force_i32) {
    if (escalated) *escalated = 0;
    if (m == 0 || n == 0) return empty_extension((uint32_t)m, out);
    orc_touch t;
    if (INITIAL_BAND >= n)
        return force_i32 ? orc_run_band(read, m, rf, n, p, 1, 0, 0, 1, 1, 0, out, &t)
                         : orc_run_dispatch(read, m, rf, n, p, 0, 0, 1, 1, 0, out, &t);
    int rc = force_i32
                 ? orc_run_band(read, m, rf, n, p, 1, 1, offset, (int64_t)num,
                                (int64_t)(den > 1 ? den : 1), INITIAL_BAND, out, &t)
                 : orc_run_dispatch(read, m, rf, n, p, 1, offset, (int64_t)num,
                                    (int64_t)(den > 1 ? den : 1), INITIAL_BAND, out, &t);
    if (rc != ORC_OK && rc != ORC_ECAP) return rc;
    int32_t perfect = (int32_t)m * p->match_score;
    if (t.touched || out->score * 20 < perfect * 17) {
        if (escalated) *escalated = 1;
        return force_i32 ? orc_run_band(read, m, rf, n, p, 1, 0, 0, 1, 1, 0, out, &t)
                         : orc_run_dispatch(read, m, rf, n, p, 0, 0, 1, 1, 0, out, &t);
    }
    return rc;
}

int orc_extend_hint(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                    const orc_params *p, int64_t offset, uint32_t num, uint32_t den,
                    orc_ext *out, int *escalated) {
    return extend_hint_impl(read, m, rf, n, p, offset, num, den, out, escalated, 0);
}

int orc_extend_hint_i32(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                        const orc_params *p, int64_t offset, uint32_t num, uint32_t den,
                        orc_ext *out, int *escalated) {
    return extend_hint_impl(read, m, rf, n, p, offset, num, den, out, escalated, 1);
}

/* Cells in the windows of rows 1..m under the band rules of :653-696. */
int64_t orc_band_cells(int64_t m, int64_t n, int has_band, int64_t offset, int64_t half) {
    if (m == 0 || n == 0) return 0;
    if (!has_band) return m * n;
    if (half < 0) half = 0;
    int64_t cells = 0;
    for (int64_t i = 1; i <= m; i++) {
        int64_t center = offset + i;
        int64_t c = center < 1 ? 1 : (center > n ? n : center);
        int64_t lo = c - half > 1 ? c - half : 1;
        int64_t hi = c + half < n ? c + half : n;
        if (hi >= lo) cells += hi - lo + 1;
    }
    return cells;
}
