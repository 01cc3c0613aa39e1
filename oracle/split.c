/*
 * split.c -- oracle restatement of the splice-rescue flank DP and its
 * helpers: crates/map/src/split.rs:150-321 (retry_tail_start,
 * build_rescue_ext, rescue_cigar_valid), :468-570 (channel_a_with_policy),
 * crates/map/src/splice.rs:63-103 (signal), :324-340 (dinuc), :864-868
 * (junction_signal), crates/map/src/span.rs:29-38 (cigar_ref_end),
 * crates/map/src/fasta.rs:77-134 (2-bit decode).  TEST INFRASTRUCTURE ONLY.
 */
#include "esp_oracle.h"

#include <stdlib.h>
#include <string.h>

/* split.rs:30 TAIL_RETRY_RADIUS, :60 TAIL_MARGIN; splice.rs:57 SPLIT_COST */
#define TAIL_RETRY_RADIUS 5
#define TAIL_MARGIN 30
#define SPLIT_COST 4

/* fasta.rs:117-134 is_n (binary search over merged N intervals) */
static int contig_is_n(const orc_contig *c, uint32_t pos) {
    uint32_t lo = 0, hi = c->n_iv_count;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        uint32_t s = c->n_iv[2 * mid], e = c->n_iv[2 * mid + 1];
        if (pos < s) hi = mid;
        else if (pos >= e) lo = mid + 1;
        else return 1;
    }
    return 0;
}

/* fasta.rs:77-116 decode_into / base: MSB-first 2-bit, N over intervals */
void orc_slice_ascii(const orc_contig *c, uint32_t start, uint32_t end, uint8_t *out) {
    static const uint8_t B[4] = {'A', 'C', 'G', 'T'};
    for (uint32_t pos = start; pos < end; pos++) {
        if (contig_is_n(c, pos)) {
            *out++ = 'N';
            continue;
        }
        uint8_t byte = c->packed[pos >> 2];
        uint32_t shift = 6 - 2 * (pos & 3);
        *out++ = B[(byte >> shift) & 3];
    }
}

/* fasta.rs:1-5 layout (N encodes as 0 in the packed bytes; callers keep N
 * as intervals). */
void orc_pack_2bit(const uint8_t *ascii, int64_t n, uint8_t *packed) {
    memset(packed, 0, (size_t)((n + 3) / 4));
    for (int64_t k = 0; k < n; k++) {
        int code = orc_base_code(ascii[k]);
        if (code > 3) code = 0;
        packed[k >> 2] |= (uint8_t)(code << (6 - 2 * (k & 3)));
    }
}

/* splice.rs:40-53 SpliceParams::default */
void orc_splice_params_default(orc_splice_params *sp) {
    sp->min_intron = 20;
    sp->max_intron = 1000000;
    sp->gt_ag_bonus = 4;
    sp->gc_ag_bonus = 2;
    sp->at_ac_bonus = 1;
    sp->noncanonical_penalty = 8;
    sp->known_bonus = 6;
    sp->refine_radius = 12;
}

static uint8_t up(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }

/* splice.rs:78-103 splice_signal */
int orc_splice_signal(const uint8_t donor[2], const uint8_t acceptor[2], int minus) {
    uint8_t d0 = up(donor[0]), d1 = up(donor[1]), a0 = up(acceptor[0]), a1 = up(acceptor[1]);
#define IS(x0, x1, s) ((x0) == (s)[0] && (x1) == (s)[1])
    if (!minus) {
        if (IS(d0, d1, "GT") && IS(a0, a1, "AG")) return ORC_SIG_GTAG;
        if (IS(d0, d1, "GC") && IS(a0, a1, "AG")) return ORC_SIG_GCAG;
        if (IS(d0, d1, "AT") && IS(a0, a1, "AC")) return ORC_SIG_ATAC;
        return ORC_SIG_NONCANON;
    }
    if (IS(d0, d1, "CT") && IS(a0, a1, "AC")) return ORC_SIG_GTAG;
    if (IS(d0, d1, "CT") && IS(a0, a1, "GC")) return ORC_SIG_GCAG;
    if (IS(d0, d1, "GT") && IS(a0, a1, "AT")) return ORC_SIG_ATAC;
    return ORC_SIG_NONCANON;
#undef IS
}

/* splice.rs:63-71 SpliceSignal::score */
int32_t orc_signal_score(int signal, const orc_splice_params *sp) {
    switch (signal) {
    case ORC_SIG_GTAG: return sp->gt_ag_bonus;
    case ORC_SIG_GCAG: return sp->gc_ag_bonus;
    case ORC_SIG_ATAC: return sp->at_ac_bonus;
    default: return -sp->noncanonical_penalty;
    }
}

/* splice.rs:324-340 dinuc */
static void dinuc(const orc_contig *c, uint32_t p, int donor, uint8_t out[2]) {
    out[0] = out[1] = 'N';
    if (!donor && p < 2) return;
    uint32_t a = donor ? p : p - 2, b = donor ? p + 2 : p;
    if ((uint64_t)a >= (uint64_t)c->len) return;
    if (b > c->len) b = c->len;
    orc_slice_ascii(c, a, b, out);
}

/* splice.rs:864-868 junction_signal */
int orc_junction_signal(const orc_contig *c, const orc_junction *j) {
    uint8_t d[2], a[2];
    dinuc(c, j->start, 1, d);
    dinuc(c, j->end, 0, a);
    return orc_splice_signal(d, a, j->minus_strand);
}

/* span.rs:29-38 cigar_ref_end (M/D/N advance; result truncated to u32) */
uint32_t orc_cigar_ref_end(uint32_t pos, const uint32_t *ops, uint32_t n_ops) {
    uint64_t r = pos;
    for (uint32_t k = 0; k < n_ops; k++) {
        uint32_t code = ops[k] & 15u;
        if (code == ORC_OP_M || code == ORC_OP_D || code == ORC_OP_N) r += ops[k] >> 4;
    }
    return (uint32_t)r;
}

static uint32_t *ext_alloc(orc_ext *e, uint32_t cap) {
    memset(e, 0, sizeof(*e));
    e->cap = cap;
    e->ops = (uint32_t *)malloc(cap * sizeof(uint32_t));
    return e->ops;
}

/* split.rs:150-223 retry_tail_start.  On return out->left/right own malloc'd
 * op buffers (release with free()) when out->found. */
int orc_retry_tail_start(const orc_contig *c, const uint8_t *read, uint32_t read_len,
                         uint32_t tail_start, const orc_junction *j, int signal,
                         uint32_t support, const orc_splice_params *sp, const orc_params *p,
                         orc_retry *out) {
    memset(out, 0, sizeof(*out));
    uint32_t lo_dro = tail_start > TAIL_RETRY_RADIUS ? tail_start - TAIL_RETRY_RADIUS : 0;
    if (lo_dro < 1) lo_dro = 1;
    uint32_t hi_dro = tail_start + TAIL_RETRY_RADIUS;
    uint32_t rl1 = read_len > 0 ? read_len - 1 : 0;
    if (hi_dro > rl1) hi_dro = rl1;
    int32_t signal_score = orc_signal_score(signal, sp);
    int32_t lib_bonus = (int32_t)((support < 10 ? support : 10) * 5);
    uint32_t cap = 2 * read_len + 8;
    orc_ext le, re;
    memset(&le, 0, sizeof(le));  /* a failed first allocation leaves re unset */
    memset(&re, 0, sizeof(re));
    uint8_t *win = (uint8_t *)malloc((size_t)read_len + 2 * TAIL_MARGIN + 8);
    if (!ext_alloc(&le, cap) || !ext_alloc(&re, cap) || !win) {
        free(le.ops); free(re.ops); free(win);
        return ORC_ENOMEM;
    }
    int rc = ORC_OK;
    for (uint32_t dro = lo_dro; dro <= hi_dro; dro++) {
        uint32_t llen = dro, rlen = read_len - dro;
        uint32_t l_hi = j->start < c->len ? j->start : c->len;
        uint32_t l_lo = l_hi > llen + TAIL_MARGIN ? l_hi - (llen + TAIL_MARGIN) : 0;
        uint32_t r_lo = j->end;
        uint64_t r_hi64 = (uint64_t)r_lo + rlen + TAIL_MARGIN;
        uint32_t r_hi = (uint32_t)(r_hi64 < c->len ? r_hi64 : c->len);
        if (l_hi <= l_lo || r_hi <= r_lo) continue;
        orc_slice_ascii(c, l_lo, l_hi, win);
        rc = orc_extend_hint(read, llen, win, l_hi - l_lo, p, 0, 1, 1, &le, NULL);
        if (rc != ORC_OK) break;
        orc_slice_ascii(c, r_lo, r_hi, win);
        rc = orc_extend_hint(read + dro, rlen, win, r_hi - r_lo, p, 0, 1, 1, &re, NULL);
        if (rc != ORC_OK) break;
        uint64_t l_al = le.read_end > le.read_start ? le.read_end - le.read_start : 0;
        uint64_t r_al = re.read_end > re.read_start ? re.read_end - re.read_start : 0;
        if (l_al * 5 < (uint64_t)llen * 4 || r_al * 5 < (uint64_t)rlen * 4) continue;
        if (le.read_end != llen || re.read_start != 0 || re.ref_start != 0 ||
            orc_cigar_ref_end(l_lo + le.ref_start, le.ops, le.n_ops) != j->start)
            continue;
        int32_t total = le.score + re.score + signal_score + lib_bonus - SPLIT_COST;
        if (!out->found || total > out->total) {
            if (out->found) {
                free(out->left.ops);
                free(out->right.ops);
            }
            out->found = 1;
            out->dro = dro;
            out->left_win_lo = l_lo;
            out->total = total;
            out->left = le;
            out->right = re;
            /* the buffers now belong to out: forget them before reallocating */
            memset(&le, 0, sizeof(le));
            memset(&re, 0, sizeof(re));
            if (!ext_alloc(&le, cap) || !ext_alloc(&re, cap)) {
                rc = ORC_ENOMEM;
                break;
            }
        }
    }
    free(le.ops);
    free(re.ops);
    free(win);
    return rc;
}

/* split.rs:282-321 rescue_cigar_valid (+ intron_chain.rs:376-385
 * cigar_conserving) */
static int rescue_cigar_valid(uint32_t pos, const uint32_t *ops, uint32_t n_ops,
                              uint32_t read_len, const orc_junction *j) {
    uint64_t total = 0;
    for (uint32_t k = 0; k < n_ops; k++) {
        uint32_t code = ops[k] & 15u;
        if (code == ORC_OP_M || code == ORC_OP_I || code == ORC_OP_S) total += ops[k] >> 4;
    }
    if (total != read_len) return 0;
    uint64_t ref = pos;
    int found = 0;
    for (uint32_t k = 0; k < n_ops; k++) {
        uint32_t code = ops[k] & 15u, n = ops[k] >> 4;
        if (n == 0) return 0;
        if (code == ORC_OP_S && k != 0 && k + 1 != n_ops) return 0;
        if (code == ORC_OP_N) {
            if (k == 0 || k + 1 == n_ops) return 0;
            if (ref == j->start && ref + n == j->end) found = 1;
            ref += n;
        } else if (code == ORC_OP_M || code == ORC_OP_D) {
            ref += n;
        }
    }
    return found && ref <= 0xFFFFFFFFull;
}

/* split.rs:468-570 channel_a_with_policy(.., either_transcript_strand =
 * false) over a caller-supplied candidate list, followed by
 * build_rescue_ext (:227-240) and rescue_cigar_valid. */
int orc_channel_a(const orc_contig *c, const uint8_t *read, uint32_t read_len,
                  uint32_t tail_start, int minus, const orc_junction *cands,
                  const uint32_t *support, uint32_t n_cands, const orc_splice_params *sp,
                  const orc_params *p, orc_rescue *out) {
    uint32_t *ocap_ops = out->ops;
    uint32_t ocap = out->cap;
    memset(out, 0, sizeof(*out));
    out->ops = ocap_ops;
    out->cap = ocap;
    orc_retry best;
    memset(&best, 0, sizeof(best));
    int best_cand = -1, best_sig = 0;
    int rc = ORC_OK;
    for (uint32_t k = 0; k < n_cands; k++) {
        const orc_junction *j = &cands[k];
        if ((j->minus_strand != 0) != (minus != 0)) continue;
        uint32_t intron = j->end - j->start;
        if (intron < sp->min_intron || intron > sp->max_intron) continue;
        int sig = orc_junction_signal(c, j);
        if (sig == ORC_SIG_NONCANON && support[k] < 2) continue;
        orc_retry o;
        rc = orc_retry_tail_start(c, read, read_len, tail_start, j, sig, support[k], sp, p, &o);
        if (rc != ORC_OK) break;
        if (!o.found) continue;
        if (best_cand < 0 || o.total > best.total) {
            if (best_cand >= 0) {
                free(best.left.ops);
                free(best.right.ops);
            }
            best = o;
            best_cand = (int)k;
            best_sig = sig;
        } else {
            free(o.left.ops);
            free(o.right.ops);
        }
    }
    if (rc != ORC_OK || best_cand < 0) {
        if (best_cand >= 0) {
            free(best.left.ops);
            free(best.right.ops);
        }
        return rc;
    }
    /* build_rescue_ext: left.cigar + N(intron) + right.cigar (push_op merge) */
    uint32_t nmax = best.left.n_ops + best.right.n_ops + 1;
    uint32_t *ops = (uint32_t *)malloc(nmax * sizeof(uint32_t));
    uint32_t n = 0;
    const orc_junction *j = &cands[best_cand];
    for (uint32_t k = 0; k < best.left.n_ops; k++) ops[n++] = best.left.ops[k];
    uint32_t intron = j->end - j->start;
#define PUSH(code, len)                                                     \
    do {                                                                    \
        if (n > 0 && (ops[n - 1] & 15u) == (code)) ops[n - 1] += (len) << 4; \
        else ops[n++] = ((len) << 4) | (code);                              \
    } while (0)
    PUSH(ORC_OP_N, intron);
    for (uint32_t k = 0; k < best.right.n_ops; k++)
        PUSH(best.right.ops[k] & 15u, best.right.ops[k] >> 4);
#undef PUSH
    uint32_t pos = best.left_win_lo + best.left.ref_start;
    if (rescue_cigar_valid(pos, ops, n, read_len, j)) {
        out->found = 1;
        out->cand = best_cand;
        out->dro = best.dro;
        out->pos = pos;
        out->score = best.total;
        out->signal = best_sig;
        out->n_ops = n;
        if (out->ops) memcpy(out->ops, ops, (n < out->cap ? n : out->cap) * sizeof(uint32_t));
        if (n > out->cap) rc = ORC_ECAP;
    }
    free(ops);
    free(best.left.ops);
    free(best.right.ops);
    return rc;
}
