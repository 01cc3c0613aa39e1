/*
 * rescore.c -- oracle restatement of the strict rescoring walk of
 * crates/map/src/align.rs:1060-1165 (Aligner::rescore_with) and
 * crates/map/src/splice.rs:119-121 (intron_length_penalty).
 * TEST INFRASTRUCTURE ONLY (see esp_oracle.h).
 */
#include <math.h>
#include <string.h>

#include "esp_oracle.h"

/* splice.rs:119-121: (8.0 * |log10(max(len, 1)) - 3|) as i32 */
int32_t orc_intron_length_penalty(uint32_t len) {
    double x = (double)(len > 1 ? len : 1);
    return (int32_t)(8.0 * fabs(log10(x) - 3.0));
}

/* extend.rs:87-93 exempt_dir: 1 = A-to-G direction (ref A / read G),
 * 0 = T-to-C (ref T / read C), -1 = an ordinary mismatch */
static int exempt_dir(uint8_t ref_b, uint8_t read_b) {
    if (ref_b == 'A' && read_b == 'G') return 1;
    if (ref_b == 'T' && read_b == 'C') return 0;
    return -1;
}

/* gtf.rs:165-169 JunctionLib::contains_any_strand: binary search of the
 * library's (contig, start, end)-sorted junctions */
static int lib_contains(const orc_lib_junction *lib, uint64_t n, uint32_t contig, uint32_t start,
                        uint32_t end) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        const orc_lib_junction *j = &lib[mid];
        int less = j->contig < contig ||
                   (j->contig == contig && (j->start < start ||
                                            (j->start == start && j->end < end)));
        int eq = j->contig == contig && j->start == start && j->end == end;
        if (eq) return 1;
        if (less) lo = mid + 1;
        else hi = mid;
    }
    return 0;
}

/* contig base as ASCII, 'N' past the end (align.rs:1073-1079) */
static uint8_t base_at(const orc_contig *c, uint32_t i) {
    uint8_t b = 'N';
    if (i < c->len) orc_slice_ascii(c, i, i + 1, &b);
    return b;
}

/* align.rs:1060-1165 rescore_with, SpliceParams::default() */
void orc_rescore(const orc_contig *c, uint32_t contig_id, uint32_t pos, const uint8_t *query,
                 uint32_t qlen, const uint32_t *ops, uint32_t n_ops, const orc_lib_junction *lib,
                 uint64_t n_lib, const orc_params *p, int dir, orc_strict *s) {
    orc_splice_params sp;
    orc_splice_params_default(&sp);
    memset(s, 0, sizeof(*s));
    int32_t score = 0;
    uint32_t ro = 0, rf = pos;
    for (uint32_t k = 0; k < n_ops; k++) {
        uint32_t n = ops[k] >> 4, op = ops[k] & 15u;
        if (op == 0) { /* Match */
            uint32_t avail = c->len > rf ? c->len - rf : 0;
            if (avail > n) avail = n;
            for (uint32_t q = 0; q < n; q++) {
                uint8_t qb = (uint64_t)ro + q < qlen ? query[ro + q] : 'N';
                uint8_t rb = q < avail ? base_at(c, rf + q) : 'N';
                if (qb == 'N' || rb == 'N') continue; /* 0 score, uncounted */
                s->aligned++;
                if (qb == rb) {
                    score += p->match_score;
                    s->matches++;
                } else {
                    int ed = exempt_dir(rb, qb);
                    int exempt = (dir == ORC_EDIT_AG && ed == 1) || (dir == ORC_EDIT_TC && ed == 0);
                    if (!exempt) score += p->mismatch;
                    if (ed == 1) s->ea_ag++;
                    else if (ed == 0) s->ea_tc++;
                    else s->mm++;
                }
            }
            ro += n;
            rf += n;
        } else if (op == 1) { /* Ins */
            score -= p->gap_open + p->gap_ext * (int32_t)n;
            s->aligned += n;
            s->ins++;
            ro += n;
        } else if (op == 2) { /* Del */
            score -= p->gap_open + p->gap_ext * (int32_t)n;
            s->aligned += n;
            s->del++;
            rf += n;
        } else if (op == 4) { /* SoftClip */
            s->clipped += n;
            ro += n;
        } else { /* RefSkip */
            int32_t before = score;
            if (lib_contains(lib, n_lib, contig_id, rf, rf + n)) {
                score += sp.known_bonus;
            } else {
                uint32_t r1 = rf == 0xffffffffu ? rf : rf + 1; /* saturating_add */
                uint32_t n2 = n >= 2 ? n - 2 : 0, n1 = n >= 1 ? n - 1 : 0;
                uint8_t donor[2] = {base_at(c, rf), base_at(c, r1)};
                uint8_t acc[2] = {base_at(c, rf + n2), base_at(c, rf + n1)};
                int32_t a = orc_signal_score(orc_splice_signal(donor, acc, 0), &sp);
                int32_t b = orc_signal_score(orc_splice_signal(donor, acc, 1), &sp);
                score += (a > b ? a : b) - orc_intron_length_penalty(n);
            }
            s->n_splice++;
            s->splice_score += score - before;
            rf += n;
        }
    }
    s->score = score;
}
