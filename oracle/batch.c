/*
 * batch.c -- multi-threaded drivers over the oracle kernels, used as the
 * timed CPU baseline.  One worker per thread with its own buffers, which is
 * how the reference spreads reads over rayon workers (crates/map/src/
 * pipeline.rs:394-403, map_init with one Aligner per worker).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "esp_oracle.h"

#include <pthread.h>

extern _Thread_local int64_t orc_tls_cells;
#include <stdlib.h>
#include <string.h>

typedef struct {
    const orc_pairs *pr;
    const orc_params *p;
    int mode;
    int64_t lo, hi;
    int32_t *score;
    uint32_t *rs, *re, *fs, *n_ops, *ops;
    uint32_t ops_stride;
    int32_t *touched;
    int64_t cells;
    int rc;
} ext_job;

static void *ext_worker(void *arg) {
    ext_job *jb = (ext_job *)arg;
    const orc_pairs *pr = jb->pr;
    jb->cells = 0;
    jb->rc = ORC_OK;
    uint32_t *tmp = NULL;
    uint32_t tmp_cap = 0;
    for (int64_t k = jb->lo; k < jb->hi; k++) {
        const uint8_t *read = pr->seqs + pr->read_off[k];
        const uint8_t *win = pr->seqs + pr->win_off[k];
        int64_t m = pr->read_len[k], n = pr->win_len[k];
        uint32_t need = (uint32_t)(2 * (m + n) + 8);
        if (need > tmp_cap) {
            free(tmp);
            tmp = (uint32_t *)malloc(need * sizeof(uint32_t));
            tmp_cap = need;
            if (!tmp) { jb->rc = ORC_ENOMEM; return NULL; }
        }
        orc_ext e = {0};
        e.ops = tmp;
        e.cap = tmp_cap;
        int rc;
        int32_t touched = 0;
        if (jb->mode == 0) {
            orc_touch t;
            int has_band = pr->half[k] >= 0;
            rc = orc_run_dispatch(read, m, win, n, jb->p, has_band, pr->offset[k], 1, 1,
                                  has_band ? pr->half[k] : 0, &e, &t);
            touched = t.touched;
            jb->cells += orc_band_cells(m, n, has_band, pr->offset[k], pr->half[k]);
        } else {
            int esc = 0;
            rc = orc_extend_hint(read, m, win, n, jb->p, pr->offset[k], 1, 1, &e, &esc);
            touched = esc;
            if (m > 0 && n > 0) {
                if (30 >= n) jb->cells += m * n;
                else {
                    jb->cells += orc_band_cells(m, n, 1, pr->offset[k], 30);
                    if (esc) jb->cells += m * n;
                }
            }
        }
        if (rc != ORC_OK) { jb->rc = rc; break; }
        jb->score[k] = e.score;
        jb->rs[k] = e.read_start;
        jb->re[k] = e.read_end;
        jb->fs[k] = e.ref_start;
        jb->n_ops[k] = e.n_ops;
        if (jb->touched) jb->touched[k] = touched;
        if (jb->ops) {
            uint32_t c = e.n_ops < jb->ops_stride ? e.n_ops : jb->ops_stride;
            memcpy(jb->ops + (size_t)k * jb->ops_stride, e.ops, c * sizeof(uint32_t));
        }
    }
    free(tmp);
    return NULL;
}

int64_t orc_batch_extend(const orc_pairs *pr, int64_t n_pairs, const orc_params *p, int mode,
                         int threads, int32_t *score, uint32_t *rs, uint32_t *re,
                         uint32_t *fs, uint32_t *n_ops, uint32_t *ops, uint32_t ops_stride,
                         int32_t *touched) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    ext_job *jobs = (ext_job *)calloc((size_t)threads, sizeof(ext_job));
    if (!tid || !jobs) { free(tid); free(jobs); return ORC_ENOMEM; }
    /* interleaved chunks keep the per-thread work balanced on mixed lengths */
    int64_t chunk = (n_pairs + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        ext_job *jb = &jobs[t];
        jb->pr = pr; jb->p = p; jb->mode = mode;
        jb->lo = (int64_t)t * chunk;
        jb->hi = jb->lo + chunk < n_pairs ? jb->lo + chunk : n_pairs;
        if (jb->lo > jb->hi) jb->lo = jb->hi;
        jb->score = score; jb->rs = rs; jb->re = re; jb->fs = fs; jb->n_ops = n_ops;
        jb->ops = ops; jb->ops_stride = ops_stride; jb->touched = touched;
        pthread_create(&tid[t], NULL, ext_worker, jb);
    }
    int64_t cells = 0;
    int rc = ORC_OK;
    for (int t = 0; t < threads; t++) {
        pthread_join(tid[t], NULL);
        cells += jobs[t].cells;
        if (jobs[t].rc != ORC_OK) rc = jobs[t].rc;
    }
    free(tid);
    free(jobs);
    return rc != ORC_OK ? rc : cells;
}

typedef struct {
    const uint8_t *seqs;
    const uint64_t *ro, *to;
    const uint32_t *rl, *tl;
    int64_t lo, hi;
    int32_t *dist;
    int64_t *end;
    int64_t cells;
    int rc;
} my_job;

static void *my_worker(void *arg) {
    my_job *jb = (my_job *)arg;
    jb->cells = 0;
    jb->rc = ORC_OK;
    for (int64_t k = jb->lo; k < jb->hi; k++) {
        int64_t m = jb->rl[k], n = jb->tl[k];
        /* The reference's callers pick the entry point by length
         * (align.rs:878-882): m <= 128 single block, else long::. */
        int rc = orc_myers_long_infix_best_end(jb->seqs + jb->ro[k], m, jb->seqs + jb->to[k],
                                               n, &jb->dist[k], &jb->end[k]);
        if (rc != ORC_OK) { jb->rc = rc; break; }
        jb->cells += m * n;
    }
    return NULL;
}

int64_t orc_batch_myers_best_end(const uint8_t *seqs, const uint64_t *read_off,
                                 const uint32_t *read_len, const uint64_t *text_off,
                                 const uint32_t *text_len, int64_t n_pairs, int threads,
                                 int32_t *dist, int64_t *end) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    my_job *jobs = (my_job *)calloc((size_t)threads, sizeof(my_job));
    if (!tid || !jobs) { free(tid); free(jobs); return ORC_ENOMEM; }
    int64_t chunk = (n_pairs + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        my_job *jb = &jobs[t];
        jb->seqs = seqs; jb->ro = read_off; jb->rl = read_len; jb->to = text_off;
        jb->tl = text_len; jb->dist = dist; jb->end = end;
        jb->lo = (int64_t)t * chunk;
        jb->hi = jb->lo + chunk < n_pairs ? jb->lo + chunk : n_pairs;
        if (jb->lo > jb->hi) jb->lo = jb->hi;
        pthread_create(&tid[t], NULL, my_worker, jb);
    }
    int64_t cells = 0;
    int rc = ORC_OK;
    for (int t = 0; t < threads; t++) {
        pthread_join(tid[t], NULL);
        cells += jobs[t].cells;
        if (jobs[t].rc != ORC_OK) rc = jobs[t].rc;
    }
    free(tid);
    free(jobs);
    return rc != ORC_OK ? rc : cells;
}

/* ---- channel A over a batch (CPU baseline of the splice configuration) ---- */
typedef struct {
    const uint8_t *garena;
    const uint64_t *cbase;
    const uint32_t *clen;
    const uint8_t *reads;       /* ASCII, concatenated */
    const uint64_t *read_off;
    const uint32_t *read_len;
    const uint32_t *tail_start;
    const uint32_t *contig;
    const uint32_t *cand_first;
    const uint32_t *cand_count;
    const uint32_t *cstart, *cend, *csupport;
    int64_t lo, hi;
    int32_t *found, *score;
    int rc;
    int64_t cells;
    orc_ca_detail *det;         /* optional per-read detail (NULL: none) */
} ca_job;

static void *ca_worker(void *arg) {
    ca_job *jb = (ca_job *)arg;
    orc_splice_params sp;
    orc_splice_params_default(&sp);
    orc_params p = {2, -4, 4, 2, ORC_EDIT_OFF};
    jb->rc = ORC_OK;
    int64_t c0 = orc_tls_cells;
    for (int64_t r = jb->lo; r < jb->hi; r++) {
        uint32_t c = jb->contig[r];
        orc_contig ctg = {jb->clen[c], jb->garena + (jb->cbase[c] >> 2), NULL, 0};
        uint32_t n = jb->cand_count[r], f = jb->cand_first[r];
        orc_junction *js = (orc_junction *)malloc((n ? n : 1) * sizeof(orc_junction));
        for (uint32_t k = 0; k < n; k++) js[k] = (orc_junction){jb->cstart[f + k], jb->cend[f + k], 0};
        uint32_t ops[1024];
        orc_rescue out = {0};
        out.ops = ops;
        out.cap = 1024;
        int rc = orc_channel_a(&ctg, jb->reads + jb->read_off[r], jb->read_len[r],
                               jb->tail_start[r], 0, js, jb->csupport + f, n, &sp, &p, &out);
        free(js);
        if (rc != ORC_OK) { jb->rc = rc; break; }
        jb->found[r] = out.found;
        jb->score[r] = out.score;
        orc_ca_detail *d = jb->det;
        if (d) {
            d->cand[r] = out.found ? out.cand : -1;
            d->dro[r] = out.dro;
            d->pos[r] = out.pos;
            d->signal[r] = out.signal;
            d->n_ops[r] = out.found ? out.n_ops : 0;
            if (out.found && d->ops) {
                uint32_t c = out.n_ops < d->ops_stride ? out.n_ops : d->ops_stride;
                memcpy(d->ops + (size_t)r * d->ops_stride, ops, c * sizeof(uint32_t));
            }
        }
    }
    jb->cells = orc_tls_cells - c0;
    return NULL;
}

int orc_batch_channel_a(const uint8_t *garena, const uint64_t *cbase, const uint32_t *clen,
                        const uint8_t *reads, const uint64_t *read_off, const uint32_t *read_len,
                        const uint32_t *tail_start, const uint32_t *contig,
                        const uint32_t *cand_first, const uint32_t *cand_count,
                        const uint32_t *cstart, const uint32_t *cend, const uint32_t *csupport,
                        int64_t n_reads, int threads, int32_t *found, int32_t *score,
                        int64_t *cells, orc_ca_detail *detail) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    ca_job *jobs = (ca_job *)calloc((size_t)threads, sizeof(ca_job));
    if (!tid || !jobs) { free(tid); free(jobs); return ORC_ENOMEM; }
    int64_t chunk = (n_reads + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        ca_job *jb = &jobs[t];
        *jb = (ca_job){garena, cbase, clen, reads, read_off, read_len, tail_start, contig,
                       cand_first, cand_count, cstart, cend, csupport, 0, 0, found, score, 0,
                       0, detail};
        jb->lo = (int64_t)t * chunk;
        jb->hi = jb->lo + chunk < n_reads ? jb->lo + chunk : n_reads;
        if (jb->lo > jb->hi) jb->lo = jb->hi;
        pthread_create(&tid[t], NULL, ca_worker, jb);
    }
    int rc = ORC_OK;
    int64_t total = 0;
    for (int t = 0; t < threads; t++) {
        pthread_join(tid[t], NULL);
        if (jobs[t].rc != ORC_OK) rc = jobs[t].rc;
        total += jobs[t].cells;
    }
    if (cells) *cells = total;
    free(tid);
    free(jobs);
    return rc;
}
