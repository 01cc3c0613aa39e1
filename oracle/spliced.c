/*
 * spliced.c -- oracle restatement of the spliced pseudo-reference DP of
 * crates/map/src/splice.rs: align_spliced (:617-664) given the exon slices
 * prepare_spliced chose (:565-607), stitch_cigar (:435-493) and
 * SplicedAlignment::genomic_start (:414-424).
 * TEST INFRASTRUCTURE ONLY (see esp_oracle.h).
 */
#include <stdlib.h>
#include <string.h>

#include "esp_oracle.h"

typedef struct {
    uint32_t *v;
    uint32_t n, cap;
    int overflow;
} outv;

/* extend.rs:254-282 push_op: merge with the previous op of the same kind */
static void push(outv *o, uint32_t code, uint32_t len) {
    if (o->n > 0 && (o->v[o->n - 1] & 15u) == code) {
        o->v[o->n - 1] += len << 4;
        return;
    }
    if (o->n < o->cap) o->v[o->n] = (len << 4) | code;
    else o->overflow = 1;
    o->n++;
}

/* splice.rs:435-493.  bounds: 3 words per exon (pseudo_start, ref_start,
 * ref_end); jlen[i]: intron length of junction i (end - start). */
uint32_t orc_stitch_cigar(const uint32_t *ops, uint32_t n_ops, uint32_t p_start,
                          const uint32_t *bounds, uint32_t n_bounds, const uint32_t *jlen,
                          uint32_t n_j, uint32_t *out, uint32_t cap) {
    outv o = {out, 0, cap, 0};
    if (n_bounds == 0) {
        for (uint32_t k = 0; k < n_ops; k++) {
            if (k < cap) out[k] = ops[k];
        }
        return n_ops;
    }
#define EXON_END(e) ((uint64_t)bounds[3 * (e)] + (uint64_t)(bounds[3 * (e) + 2] - bounds[3 * (e) + 1]))
    uint64_t p = p_start;
    uint32_t ei = 0;
    while (ei + 1 < n_bounds && p >= EXON_END(ei)) ei++;
    for (uint32_t k = 0; k < n_ops; k++) {
        uint32_t code = ops[k] & 15u, len = ops[k] >> 4;
        if (code == ORC_OP_I || code == ORC_OP_S || code == ORC_OP_N) {
            push(&o, code, len);
            continue;
        }
        uint64_t remaining = len;
        while (remaining > 0) {
            if (ei >= n_bounds) {
                push(&o, code, (uint32_t)remaining);
                p += remaining;
                break;
            }
            if (p < bounds[3 * ei]) p = bounds[3 * ei]; /* snap into the exon slice */
            uint64_t end = EXON_END(ei);
            uint64_t in_exon = end > p ? end - p : 0;
            uint64_t take = remaining < in_exon ? remaining : in_exon;
            if (take > 0) push(&o, code, (uint32_t)take);
            p += take;
            remaining -= take;
            if (remaining > 0) {
                if (ei + 1 >= n_bounds) {
                    push(&o, code, (uint32_t)remaining);
                    p += remaining;
                    break;
                }
                if (ei < n_j) push(&o, ORC_OP_N, jlen[ei]);
                ei++;
            }
        }
    }
#undef EXON_END
    return o.n;
}

/* splice.rs:414-424 genomic_start */
uint32_t orc_genomic_start(uint32_t p, const uint32_t *bounds, uint32_t n_bounds) {
    for (uint32_t e = 0; e < n_bounds; e++) {
        uint32_t ps = bounds[3 * e], rs = bounds[3 * e + 1], re = bounds[3 * e + 2];
        if (p >= ps && p < ps + (re - rs)) return rs + (p - ps);
    }
    uint32_t ps = bounds[3 * (n_bounds - 1)], rs = bounds[3 * (n_bounds - 1) + 1];
    return rs + (p > ps ? p - ps : 0);
}

/* splice.rs:617-664 align_spliced after prepare_spliced: the pseudo-reference
 * is the concatenation of the exon slices [rs, re) (N for N runs), the DP is
 * extend_hint along the direct diagonal, the CIGAR is stitched back with an
 * intron of exons[i+1].rs - exons[i].re at every seam. */
int orc_align_spliced_exons(const orc_contig *c, const uint8_t *read, uint32_t m,
                            const uint32_t *exons, uint32_t n_exons, const orc_params *p,
                            orc_ext *ext, uint32_t *stitched, uint32_t cap,
                            uint32_t *n_stitched, uint32_t *gstart) {
    uint64_t total = 0;
    for (uint32_t e = 0; e < n_exons; e++) total += exons[2 * e + 1] - exons[2 * e];
    uint8_t *pseudo = (uint8_t *)malloc(total ? total : 1);
    uint32_t *bounds = (uint32_t *)calloc(3 * (size_t)(n_exons ? n_exons : 1), sizeof(uint32_t));
    uint32_t *jl = (uint32_t *)calloc(n_exons ? n_exons : 1, sizeof(uint32_t));
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (2 * (m + total) + 8));
    if (!pseudo || !bounds || !jl || !tmp) {
        free(pseudo), free(bounds), free(jl), free(tmp);
        return ORC_ENOMEM;
    }
    uint64_t at = 0;
    for (uint32_t e = 0; e < n_exons; e++) {
        uint32_t rs = exons[2 * e], re = exons[2 * e + 1];
        bounds[3 * e] = (uint32_t)at;
        bounds[3 * e + 1] = rs;
        bounds[3 * e + 2] = re;
        orc_slice_ascii(c, rs, re, pseudo + at);
        at += re - rs;
        if (e + 1 < n_exons) jl[e] = exons[2 * (e + 1)] - re;
    }
    orc_ext x = *ext;
    x.ops = tmp;
    x.cap = (uint32_t)(2 * (m + total) + 8);
    int rc = orc_extend_hint(read, m, pseudo, (int64_t)total, p, 0, 1, 1, &x, NULL);
    if (rc == ORC_OK) {
        *n_stitched = orc_stitch_cigar(tmp, x.n_ops, x.ref_start, bounds, n_exons, jl,
                                       n_exons ? n_exons - 1 : 0, stitched, cap);
        *gstart = n_exons ? orc_genomic_start(x.ref_start, bounds, n_exons) : 0;
        uint32_t k = x.n_ops < ext->cap ? x.n_ops : ext->cap;
        if (ext->ops && k) memcpy(ext->ops, tmp, k * sizeof(uint32_t));
        ext->read_start = x.read_start;
        ext->read_end = x.read_end;
        ext->ref_start = x.ref_start;
        ext->score = x.score;
        ext->n_ops = x.n_ops;
    }
    free(pseudo), free(bounds), free(jl), free(tmp);
    return rc;
}
