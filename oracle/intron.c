/*
 * intron.c -- oracle restatement of the intron-chain fast path of
 * crates/map/src/intron_chain.rs from the best fragment pair on
 * (try_intron_chain_placement :392-538): the EA-Myers breakpoint refinement
 * (refine_donor_end / refine_acceptor_start :285-343), the split-read
 * verification (verify_split_read :347-373), the read-aware junction
 * refinement (splice.rs:208-313 refine_junction_read), the pseudo-reference
 * extend_hint and stitch_cigar, and the gates between them.
 * TEST INFRASTRUCTURE ONLY (see esp_oracle.h).
 */
#include <limits.h>
#include <stdlib.h>
#include <string.h>

#include "esp_oracle.h"

#define MIN_INTRON 20 /* intron_chain.rs:47 */

static int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
static int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

/* intron_chain.rs:285-312 refine_donor_end */
uint32_t orc_refine_donor_end(const orc_contig *c, const uint8_t *read, uint32_t len,
                              uint32_t junction_off, uint32_t frag_ref_hi,
                              int64_t frag_implied_start, uint32_t refine_window,
                              uint32_t pattern_len) {
    int64_t w = refine_window;
    uint32_t off = junction_off < len ? junction_off : len;
    uint32_t lo = (uint32_t)max64((int64_t)frag_ref_hi - w, 0);
    uint32_t hi = (uint32_t)min64((int64_t)frag_ref_hi + w, (int64_t)c->len);
    uint32_t fallback = frag_ref_hi ? frag_ref_hi - 1 : 0;
    if (hi <= lo || off == 0) return fallback;
    uint32_t text_lo_in_read = (uint32_t)max64((int64_t)lo - frag_implied_start + 2, 0);
    uint32_t pat_start = off > pattern_len ? off - pattern_len : 0;
    if (pat_start < text_lo_in_read) pat_start = text_lo_in_read;
    if (pat_start >= off) return fallback;
    uint8_t *text = (uint8_t *)malloc(hi - lo);
    if (!text) return fallback;
    orc_slice_ascii(c, lo, hi, text);
    int32_t dist;
    int64_t end = 0;
    orc_myers_infix_best_end(read + pat_start, off - pat_start, text, hi - lo, &dist, &end);
    free(text);
    return lo + (uint32_t)end;
}

/* intron_chain.rs:314-343 refine_acceptor_start */
uint32_t orc_refine_acceptor_start(const orc_contig *c, const uint8_t *read, uint32_t len,
                                   uint32_t junction_off, uint32_t frag_ref_lo,
                                   int64_t frag_implied_start, uint32_t refine_window,
                                   uint32_t pattern_len) {
    int64_t w = refine_window;
    uint32_t off = junction_off < len ? junction_off : len;
    uint32_t lo = (uint32_t)max64((int64_t)frag_ref_lo - w, 0);
    uint32_t hi = (uint32_t)min64((int64_t)frag_ref_lo + w, (int64_t)c->len);
    if (hi <= lo) return frag_ref_lo;
    uint64_t text_hi_in_read = (uint64_t)max64((int64_t)hi - frag_implied_start - 2, 0);
    uint64_t pat_end = (uint64_t)off + pattern_len;
    if (pat_end > len) pat_end = len;
    if (pat_end > text_hi_in_read) pat_end = text_hi_in_read;
    if (pat_end <= off) return frag_ref_lo;
    uint8_t *text = (uint8_t *)malloc(hi - lo);
    if (!text) return frag_ref_lo;
    orc_slice_ascii(c, lo, hi, text);
    int32_t dist;
    int64_t start = 0;
    orc_myers_infix_best_start(read + off, (int64_t)(pat_end - off), text, hi - lo, &dist,
                               &start);
    free(text);
    return lo + (uint32_t)start;
}

/* intron_chain.rs:347-373 verify_split_read; frag offsets are
 * off_lo = r_lo - q_lo (intron_chain.rs:104-106). */
void orc_verify_split_read(const orc_contig *c, const uint8_t *read, uint32_t len,
                           int64_t left_off_lo, uint32_t right_r_hi, int64_t donor_end,
                           int64_t acceptor_start, int32_t *vd, int32_t *va) {
    *vd = *va = INT32_MAX;
    uint32_t mid = len / 2;
    int64_t clen = c->len;
    uint32_t d_start = (uint32_t)max64(left_off_lo - 30, 0);
    uint32_t d_end = (uint32_t)min64(max64(donor_end + 1 + 30, 1), clen);
    uint32_t a_start = (uint32_t)min64(max64(acceptor_start - 30, 0), clen);
    uint32_t a_end = (uint32_t)min64(max64((int64_t)right_r_hi + 30, (int64_t)a_start + 1), clen);
    if (d_start >= d_end || a_start >= a_end || mid == 0 || mid >= len) return;
    uint8_t *dt = (uint8_t *)malloc(d_end - d_start), *at = (uint8_t *)malloc(a_end - a_start);
    if (!dt || !at) {
        free(dt), free(at);
        return;
    }
    orc_slice_ascii(c, d_start, d_end, dt);
    orc_slice_ascii(c, a_start, a_end, at);
    orc_myers_long_infix(read, mid, dt, d_end - d_start, vd);
    orc_myers_long_infix(read + mid, len - mid, at, a_end - a_start, va);
    free(dt), free(at);
}

/* gtf.rs:142-149 JunctionLib::support: exact (contig, start, end, strand) */
uint32_t orc_lib_support(const orc_lib_entry *lib, uint64_t n, uint32_t contig, uint32_t start,
                         uint32_t end, int minus) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        const orc_lib_entry *x = &lib[mid];
        int less = x->contig != contig ? x->contig < contig
                   : x->start != start ? x->start < start
                   : x->end != end     ? x->end < end
                                       : (x->minus != 0) < (minus != 0);
        int eq = x->contig == contig && x->start == start && x->end == end &&
                 (x->minus != 0) == (minus != 0);
        if (eq) return x->count;
        if (less) lo = mid + 1;
        else hi = mid;
    }
    return 0;
}

/* fasta.rs:30-38 Base::from_ascii codes: A C G T = 0..3, other = 4 (N) */
static int base_code(uint8_t b) {
    switch (b) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

/* splice.rs:316-321 edit_equiv: equal, or A<->G / T<->C */
static int edit_equiv(int a, int b) {
    return a == b || (a == 0 && b == 2) || (a == 2 && b == 0) || (a == 3 && b == 1) ||
           (a == 1 && b == 3);
}

static int contig_base(const orc_contig *c, uint32_t pos) {
    uint8_t b;
    orc_slice_ascii(c, pos, pos + 1, &b);
    return base_code(b);
}

static void dinuc_of(const orc_contig *c, uint32_t p, int donor, uint8_t out[2]) {
    out[0] = out[1] = 'N';
    if (!donor && p < 2) return;
    uint32_t a = donor ? p : p - 2, b = donor ? p + 2 : p;
    if ((uint64_t)a >= (uint64_t)c->len) return;
    if (b > c->len) b = c->len;
    orc_slice_ascii(c, a, b, out);
}

/* splice.rs:208-313 refine_junction_read; returns 1 and the junction when a
 * boundary exists. */
int orc_refine_junction_read(const orc_contig *c, uint32_t contig_id, const uint8_t *read,
                             uint32_t read_len, uint32_t naive_start, uint32_t naive_end,
                             uint32_t q_a, uint32_t q_b, int minus, const orc_lib_entry *lib,
                             uint64_t n_lib, const orc_splice_params *sp, orc_junction *out,
                             int *signal, uint32_t *support) {
    int64_t len = c->len;
    int64_t ref_gap = (int64_t)naive_end - (int64_t)naive_start;
    int64_t read_gap = (int64_t)q_b - (int64_t)q_a;
    if (read_gap > 20) return 0;
    int64_t intron_len = ref_gap - read_gap;
    if (intron_len < (int64_t)sp->min_intron || intron_len > (int64_t)sp->max_intron) return 0;
    int64_t margin = 2;
    int64_t lo = (read_gap < 0 ? read_gap : 0) - margin;
    int64_t hi = (read_gap > 0 ? read_gap : 0) + margin;
    int have = 0;
    int32_t best = 0;
    for (int64_t delta = lo; delta <= hi; delta++) {
        int64_t s = (int64_t)naive_start + delta;
        if (s < 0) continue;
        int64_t e = s + intron_len;
        if (e < 2 || e > len) continue;
        int64_t qb = (int64_t)q_a + delta;
        if (qb < 1 || (uint64_t)qb >= read_len) continue;
        int32_t m = 0;
        for (int64_t i = 1; i <= 4; i++) {
            int64_t q1 = qb - i, g1 = s - i;
            if (q1 >= 0 && g1 >= 0 &&
                edit_equiv(base_code(read[q1]), contig_base(c, (uint32_t)g1)))
                m++;
            int64_t q2 = qb + i - 1, g2 = e + i - 1;
            if ((uint64_t)q2 < read_len && g2 < len &&
                edit_equiv(base_code(read[q2]), contig_base(c, (uint32_t)g2)))
                m++;
        }
        for (int t = 0; t < 2; t++) {
            int tm = t == 0 ? minus : !minus;
            uint8_t d[2], a[2];
            dinuc_of(c, (uint32_t)s, 1, d);
            dinuc_of(c, (uint32_t)e, 0, a);
            int sig = orc_splice_signal(d, a, tm);
            uint32_t sup = orc_lib_support(lib, n_lib, contig_id, (uint32_t)s, (uint32_t)e, tm);
            int64_t ad = delta < 0 ? -delta : delta;
            int32_t score = m * 50 + orc_signal_score(sig, sp) * 5 - (int32_t)ad * 5;
            if (sup > 0) score += sp->known_bonus;
            if (!have || score > best) {
                have = 1;
                best = score;
                out->start = (uint32_t)s;
                out->end = (uint32_t)e;
                out->minus_strand = tm;
                *signal = sig;
                *support = sup;
            }
        }
    }
    return have;
}

/* intron_chain.rs:376-386 cigar_conserving: M/I/S consume the read exactly */
static int cigar_conserving(const uint32_t *ops, uint32_t n, uint32_t read_len) {
    uint64_t t = 0;
    for (uint32_t k = 0; k < n; k++) {
        uint32_t code = ops[k] & 15u;
        if (code == ORC_OP_M || code == ORC_OP_I || code == ORC_OP_S) t += ops[k] >> 4;
    }
    return t == read_len;
}

/* intron_chain.rs:392-538 after best_frag_pair: everything from the
 * junction offset on.  Returns ORC_OK with out->found = 0 when a stage
 * rejects (out->stage names it) or 1 with the spliced alignment. */
int orc_intron_chain(const orc_contig *c, uint32_t contig_id, const uint8_t *read,
                     uint32_t len, const orc_frag *left, const orc_frag *right,
                     uint32_t pair_intron_start, uint32_t pair_intron_end, int minus,
                     const orc_lib_entry *lib, uint64_t n_lib, const orc_intron_params *ip,
                     const orc_params *p, orc_intron_out *out) {
    uint32_t *keep_ops = out->ext.ops, keep_cap = out->ext.cap;
    uint32_t *keep_st = out->stitched;
    uint32_t st_cap = out->stitched_cap;
    memset(out, 0, sizeof(*out));
    out->ext.ops = keep_ops;
    out->ext.cap = keep_cap;
    out->stitched = keep_st;
    out->stitched_cap = st_cap;
    out->vd = out->va = INT32_MAX;
    if (len == 0) {
        out->stage = ORC_IC_EMPTY;
        return ORC_OK;
    }
    int64_t left_off = (int64_t)left->r_lo - (int64_t)left->q_lo;
    int64_t right_off = (int64_t)right->r_lo - (int64_t)right->q_lo;
    uint32_t j_est = len / 2;
    uint32_t junction_off = j_est;
    if (left->q_hi < right->q_lo)
        junction_off = j_est < left->q_hi ? left->q_hi : (j_est > right->q_lo ? right->q_lo : j_est);
    int64_t donor_end = orc_refine_donor_end(c, read, len, junction_off, left->r_hi, left_off,
                                             ip->refine_window, ip->refine_pattern_len);
    int64_t acceptor_start = orc_refine_acceptor_start(c, read, len, junction_off, right->r_lo,
                                                       right_off, ip->refine_window,
                                                       ip->refine_pattern_len);
    int64_t intron_len = acceptor_start - donor_end - 1;
    out->donor_end = (uint32_t)donor_end;
    out->acceptor_start = (uint32_t)acceptor_start;
    orc_verify_split_read(c, read, len, left_off, right->r_hi, donor_end, acceptor_start,
                          &out->vd, &out->va);
    uint32_t total_anchors = left->n_anchors + right->n_anchors;
    int64_t max_v = out->vd > out->va ? out->vd : out->va;
    int64_t sum_v = (int64_t)out->vd + out->va;
    int32_t max_t = (int32_t)((double)len * 0.17), sum_t = (int32_t)((double)len * 0.24);
    if (total_anchors < 2) {
        out->stage = ORC_IC_ANCHORS;
        return ORC_OK;
    }
    if (intron_len < MIN_INTRON || intron_len > (int64_t)ip->intron_max) {
        out->stage = ORC_IC_INTRON;
        return ORC_OK;
    }
    if (max_v > max_t || sum_v > sum_t) {
        out->stage = ORC_IC_VERIFY;
        return ORC_OK;
    }
    orc_splice_params sp;
    orc_splice_params_default(&sp);
    sp.max_intron = ip->intron_max;
    orc_junction j;
    int sig;
    uint32_t sup;
    if (!orc_refine_junction_read(c, contig_id, read, len, left->r_hi, right->r_lo, left->q_hi,
                                  right->q_lo, minus, lib, n_lib, &sp, &j, &sig, &sup)) {
        j.start = pair_intron_start;
        j.end = pair_intron_end;
        j.minus_strand = minus;
        sup = orc_lib_support(lib, n_lib, contig_id, j.start, j.end, minus);
        sig = orc_junction_signal(c, &j);
    }
    out->junction = j;
    out->signal = sig;
    out->support = sup;
    if (j.end <= j.start || j.end - j.start < MIN_INTRON || j.end - j.start > ip->intron_max) {
        out->stage = ORC_IC_JUNCTION;
        return ORC_OK;
    }
    uint32_t left_start = left->r_lo > len ? left->r_lo - len : 0;
    uint64_t re = (uint64_t)right->r_hi + len;
    uint32_t right_end = (uint32_t)(re < c->len ? re : c->len);
    if (left_start >= j.start || j.end >= right_end) {
        out->stage = ORC_IC_BOUNDS;
        return ORC_OK;
    }
    out->left_start = left_start;
    out->right_end = right_end;
    uint32_t total = (j.start - left_start) + (right_end - j.end);
    uint8_t *pseudo = (uint8_t *)malloc(total);
    uint32_t cap = 2 * (len + total) + 8;
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * cap);
    if (!pseudo || !tmp) {
        free(pseudo), free(tmp);
        return ORC_ENOMEM;
    }
    orc_slice_ascii(c, left_start, j.start, pseudo);
    orc_slice_ascii(c, j.end, right_end, pseudo + (j.start - left_start));
    orc_ext x = {0};
    x.ops = tmp;
    x.cap = cap;
    int rc = orc_extend_hint(read, len, pseudo, total, p, left_off - (int64_t)left_start, 1, 1,
                             &x, NULL);
    if (rc != ORC_OK) {
        free(pseudo), free(tmp);
        return rc;
    }
    uint32_t bounds[6] = {0, left_start, j.start, j.start - left_start, j.end, right_end};
    uint32_t jl = j.end - j.start;
    uint32_t *st = (uint32_t *)malloc(sizeof(uint32_t) * (cap + 4));
    if (!st) {
        free(pseudo), free(tmp);
        return ORC_ENOMEM;
    }
    uint32_t ns = orc_stitch_cigar(tmp, x.n_ops, x.ref_start, bounds, 2, &jl, 1, st, cap + 4);
    out->ext.read_start = x.read_start;
    out->ext.read_end = x.read_end;
    out->ext.ref_start = x.ref_start;
    out->ext.score = x.score;
    out->ext.n_ops = x.n_ops;
    if (out->ext.ops)
        memcpy(out->ext.ops, tmp, sizeof(uint32_t) * (x.n_ops < out->ext.cap ? x.n_ops : out->ext.cap));
    out->n_stitched = ns;
    if (out->stitched)
        memcpy(out->stitched, st, sizeof(uint32_t) * (ns < out->stitched_cap ? ns : out->stitched_cap));
    int has_n = 0;
    for (uint32_t k = 0; k < ns; k++) has_n |= (st[k] & 15u) == ORC_OP_N;
    if (x.score <= 0 || !cigar_conserving(st, ns, len) || !has_n) {
        out->stage = ORC_IC_RESULT;
    } else {
        out->found = 1;
        out->stage = ORC_IC_FOUND;
    }
    free(pseudo), free(tmp), free(st);
    return ORC_OK;
}
