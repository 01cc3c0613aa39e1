// abi_splice.cu -- C ABI of the resident genome and the splice-rescue flank
// DP (split.rs retry_tail_start and channel A).
#include <cuda_runtime.h>

#include <new>

#include "esp_host.h"

namespace {

struct SpliceBufs {
    esp::SpliceItem *items;
    esp::SpliceItemOut *item_out;
    int32_t *read_status;
    esp_pair *dp_pairs;
    esp_n_interval *dp_iv;
    esp_extension *dp_out;
    uint32_t *dp_cig;
    unsigned long long *cells;
};

constexpr uint32_t DP_STRIDE = 48;  // CIGAR ops per segment extension

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

// Device scratch of one splice batch with n_cands candidates.
int splice_scratch(esp_handle *h, uint64_t n_reads, uint64_t n_cands, bool any_n, SpliceBufs &B) {
    const uint64_t slots = n_cands * esp::SPL_SLOTS;
    size_t s_items = al256(n_cands * sizeof(esp::SpliceItem));
    size_t s_io = al256(n_cands * sizeof(esp::SpliceItemOut));
    size_t s_rs = al256(n_reads * sizeof(int32_t));
    size_t s_pairs = al256(slots * sizeof(esp_pair));
    size_t s_iv = any_n ? al256(slots * esp::SPL_IVCAP * sizeof(esp_n_interval)) : 0;
    size_t s_out = al256(slots * sizeof(esp_extension));
    size_t s_cig = al256(slots * DP_STRIDE * sizeof(uint32_t));
    size_t total = s_items + s_io + s_rs + s_pairs + s_iv + s_out + s_cig + 256;
    int rc = grow_device(h, &h->d_spl, &h->d_spl_cap, total);
    if (rc != ESP_OK) return rc;
    uint8_t *p = (uint8_t *)h->d_spl;
    B.items = (esp::SpliceItem *)p;
    p += s_items;
    B.item_out = (esp::SpliceItemOut *)p;
    p += s_io;
    B.read_status = (int32_t *)p;
    p += s_rs;
    B.dp_pairs = (esp_pair *)p;
    p += s_pairs;
    B.dp_iv = any_n ? (esp_n_interval *)p : nullptr;
    p += s_iv;
    B.dp_out = (esp_extension *)p;
    p += s_out;
    B.dp_cig = (uint32_t *)p;
    p += s_cig;
    B.cells = (unsigned long long *)p;
    return ESP_OK;
}

// Enqueue build -> DP (extend_hint) -> select for a device-resident batch.
int enqueue_splice(esp_handle *h, const esp_genome *g, const esp_splice_read *d_reads,
                   uint64_t n_reads, uint32_t max_read_len, const uint8_t *d_read_arena,
                   uint64_t read_arena_bytes, const esp_n_interval *d_read_iv,
                   uint64_t read_iv_count, const esp_splice_cand *d_cands, uint64_t n_cands,
                   const esp_splice_params &sp, const esp::GotohConst &K, esp_splice_result *d_out,
                   uint32_t *d_cigar, uint32_t cigar_stride, cudaStream_t st, bool retry_only,
                   int forced_signal, SpliceBufs &B) {
    const bool any_n = read_iv_count > 0 || g->n_iv > 0;
    int rc = splice_scratch(h, n_reads, n_cands, any_n, B);
    if (rc != ESP_OK) return rc;
    esp::SpliceJob J{};
    J.retry_only = retry_only ? 1 : 0;
    J.forced_signal = forced_signal;
    J.item_out = B.item_out;
    J.reads = d_reads;
    J.n_reads = n_reads;
    J.read_arena = d_read_arena;
    J.read_iv = d_read_iv;
    J.g_arena = g->d_arena;
    J.contigs = g->d_contigs;
    J.n_contigs = (uint32_t)g->contigs.size();
    J.g_iv = g->d_iv;
    J.cands = d_cands;
    J.sp = sp;
    J.items = B.items;
    J.read_status = B.read_status;
    J.dp_pairs = B.dp_pairs;
    J.dp_iv = B.dp_iv;
    J.dp_out = B.dp_out;
    J.dp_cig = B.dp_cig;
    J.dp_stride = DP_STRIDE;
    J.out = d_out;
    J.cigar = d_cigar;
    J.cigar_stride = cigar_stride;
    CK(h, esp::launch_splice_build(J, h->num_sms, st));
    uint64_t launches = 1;
    const uint64_t slots = n_cands * esp::SPL_SLOTS;
    Limits L1, L2;
    add_limits(L1, max_read_len, max_read_len + 30, 30);
    add_limits(L2, max_read_len, max_read_len + 30, -1);
    rc = enqueue_batch(h, ESP_MODE_HINT, B.dp_pairs, slots, d_read_arena, read_arena_bytes, B.dp_iv,
                       any_n ? slots * esp::SPL_IVCAP : 0, K, L1, L2, B.dp_out, B.dp_cig,
                       DP_STRIDE, st, g->d_arena, g->arena_bytes);
    if (rc != ESP_OK) return rc;
    launches += h->launches;
    CK(h, esp::launch_splice_select(J, h->num_sms, st));
    h->launches = launches + 1;
    return ESP_OK;
}

}  // namespace

extern "C" {

int esp_genome_create(esp_handle *h, const uint8_t *arena, uint64_t arena_bytes,
                      const esp_contig *contigs, uint32_t n_contigs,
                      const esp_n_interval *n_iv, uint64_t n_iv_count, esp_genome **out) {
    if (!h || !out || !arena || (n_contigs && !contigs) || (n_iv_count && !n_iv))
        return fail(h, ESP_EINVAL, "null argument");
    *out = nullptr;
    for (uint32_t c = 0; c < n_contigs; c++) {
        const esp_contig &C = contigs[c];
        if (C.base + C.len > arena_bytes * 4 || (uint64_t)C.n_first + C.n_count > n_iv_count)
            return fail(h, ESP_EINVAL, "contig outside the arena or the N table");
    }
    CK(h, cudaSetDevice(h->device));
    esp_genome *g = new (std::nothrow) esp_genome();
    if (!g) return fail(h, ESP_ENOMEM, "genome");
    g->device = h->device;
    g->arena_bytes = arena_bytes;
    g->contigs.assign(contigs, contigs + n_contigs);
    g->n_iv = n_iv_count;
    if (n_iv_count) g->h_iv.assign(n_iv, n_iv + n_iv_count);
    cudaError_t e = cudaMalloc((void **)&g->d_arena, arena_bytes + 16);
    if (e == cudaSuccess) e = cudaMalloc((void **)&g->d_contigs, std::max<size_t>(1, n_contigs) * sizeof(esp_contig));
    if (e == cudaSuccess) e = cudaMalloc((void **)&g->d_iv, std::max<size_t>(1, n_iv_count) * sizeof(esp_n_interval));
    if (e == cudaSuccess) e = cudaMemcpy(g->d_arena, arena, arena_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g->d_arena + arena_bytes, 0, 16);
    if (e == cudaSuccess && n_contigs)
        e = cudaMemcpy(g->d_contigs, contigs, n_contigs * sizeof(esp_contig), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_iv_count)
        e = cudaMemcpy(g->d_iv, n_iv, n_iv_count * sizeof(esp_n_interval), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        esp_genome_destroy(g);
        return cuda_fail(h, e, "esp_genome_create");
    }
    *out = g;
    return ESP_OK;
}

int esp_genome_destroy(esp_genome *g) {
    if (!g) return ESP_OK;
    cudaSetDevice(g->device);
    cudaFree(g->d_arena);
    cudaFree(g->d_contigs);
    cudaFree(g->d_iv);
    delete g;
    return ESP_OK;
}

uint64_t esp_last_cells(const esp_handle *h) { return h ? h->last_cells : 0; }

int esp_retry_tail_start(esp_handle *h, const esp_genome *g, const uint8_t *read, size_t read_len,
                         uint32_t tail_start, const esp_junction *j, int signal,
                         uint32_t support, const esp_splice_params *sp,
                         const esp_extend_params *params, esp_retry_outcome *out,
                         uint32_t *left_cigar, uint32_t *right_cigar, uint32_t cigar_cap) {
    if (!h || !g || !j || !sp || !params || !out || (read_len && !read))
        return fail(h, ESP_EINVAL, "null argument");
    if (read_len > 32767) return fail(h, ESP_EDOMAIN, "read longer than 32767");
    if (signal < 0 || signal > 3) return fail(h, ESP_EINVAL, "bad splice signal");
    memset(out, 0, sizeof(*out));
    if (j->contig >= g->contigs.size()) return ESP_OK;  // reference.contigs.get(..)? -> None
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    CK(h, cudaSetDevice(h->device));
    // staging: read record | candidate | N intervals | read arena
    std::vector<esp_n_interval> iv;
    size_t arena_bytes = ((read_len + 3) / 4 + 15) / 16 * 16 + 16;
    size_t off_cand = 256, off_iv = 512, off_arena = al256(off_iv + 8 * (read_len / 2 + 2));
    size_t off_res = al256(off_arena + arena_bytes);
    size_t total = off_res + 256;
    int rc;
    if ((rc = grow_host(h, &h->h_in, &h->h_in_cap, total)) != ESP_OK) return rc;
    if ((rc = grow_device(h, &h->d_spl_io, &h->d_spl_io_cap, total)) != ESP_OK) return rc;
    uint8_t *hb = (uint8_t *)h->h_in;
    memset(hb, 0, total);
    encode_seq(read, read_len, hb + off_arena, 0, iv);
    esp_splice_read R{};
    R.read_pos = 0;
    R.read_len = (uint32_t)read_len;
    R.tail_start = tail_start;
    R.contig = j->contig;
    R.minus = j->minus_strand;
    R.cand_first = 0;
    R.cand_count = 1;
    R.n_first = 0;
    R.n_read = (uint32_t)iv.size();
    esp_splice_cand cd{*j, support};
    memcpy(hb, &R, sizeof(R));
    memcpy(hb + off_cand, &cd, sizeof(cd));
    if (!iv.empty()) memcpy(hb + off_iv, iv.data(), iv.size() * sizeof(esp_n_interval));
    uint8_t *db = (uint8_t *)h->d_spl_io;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(db, hb, off_res, cudaMemcpyHostToDevice, st));
    SpliceBufs B;
    uint32_t dummy_stride = 1;
    rc = enqueue_splice(h, g, (const esp_splice_read *)db, 1, (uint32_t)std::max<size_t>(read_len, 1),
                        db + off_arena, arena_bytes, iv.empty() ? nullptr : (const esp_n_interval *)(db + off_iv),
                        iv.size(), (const esp_splice_cand *)(db + off_cand), 1, *sp, K,
                        (esp_splice_result *)(db + off_res), (uint32_t *)(db + off_res + 64),
                        dummy_stride, st, true, signal, B);
    if (rc != ESP_OK) return rc;
    esp::SpliceItemOut io;
    CK(h, cudaMemcpyAsync(&io, B.item_out, sizeof(io), cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    int32_t rstat = 0;
    CK(h, cudaMemcpy(&rstat, B.read_status, sizeof(rstat), cudaMemcpyDeviceToHost));
    if (rstat != ESP_OK) return fail(h, rstat, "splice retry refused (N runs)");
    if (!io.found) return ESP_OK;
    esp_extension ext[2];
    CK(h, cudaMemcpy(ext, B.dp_out + io.slot, sizeof(ext), cudaMemcpyDeviceToHost));
    out->found = 1;
    out->dro = io.dro;
    out->left_win_lo = io.left_win_lo;
    out->total = io.total;
    out->left = ext[0];
    out->right = ext[1];
    if (ext[0].n_ops > cigar_cap || ext[1].n_ops > cigar_cap)
        return fail(h, ESP_ECAP, "CIGAR buffer too small");
    if (left_cigar && ext[0].n_ops)
        CK(h, cudaMemcpy(left_cigar, B.dp_cig + io.slot * DP_STRIDE, ext[0].n_ops * 4,
                         cudaMemcpyDeviceToHost));
    if (right_cigar && ext[1].n_ops)
        CK(h, cudaMemcpy(right_cigar, B.dp_cig + (io.slot + 1) * DP_STRIDE, ext[1].n_ops * 4,
                         cudaMemcpyDeviceToHost));
    return ESP_OK;
}

int esp_batch_splice_host(esp_handle *h, const esp_genome *g, const esp_splice_read *reads,
                          uint64_t n_reads, const uint8_t *read_arena, uint64_t read_arena_bytes,
                          const esp_n_interval *read_n_iv, uint64_t read_n_iv_count,
                          const esp_splice_cand *cands, uint64_t n_cands,
                          const esp_splice_params *sp, const esp_extend_params *params,
                          esp_splice_result *out, uint32_t *cigar, uint32_t cigar_stride) {
    if (!h || !g || !sp || !params || !out || (n_reads && (!reads || !read_arena)) ||
        (n_cands && !cands))
        return fail(h, ESP_EINVAL, "null argument");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    uint32_t maxL = 1;
    for (uint64_t r = 0; r < n_reads; r++) {
        const esp_splice_read &R = reads[r];
        if (R.read_len > 32767 || (uint64_t)R.cand_first + R.cand_count > n_cands ||
            R.read_pos + R.read_len > read_arena_bytes * 4 ||
            (uint64_t)R.n_first + R.n_read > read_n_iv_count)
            return fail(h, ESP_EINVAL, "read record outside its tables");
        maxL = std::max(maxL, R.read_len);
    }
    CK(h, cudaSetDevice(h->device));
    size_t s_r = al256(n_reads * sizeof(esp_splice_read));
    size_t s_a = al256(read_arena_bytes + 16);
    size_t s_iv = al256(read_n_iv_count * sizeof(esp_n_interval));
    size_t s_c = al256(n_cands * sizeof(esp_splice_cand));
    size_t s_o = al256(n_reads * sizeof(esp_splice_result));
    size_t s_g = al256(n_reads * (size_t)cigar_stride * 4);
    int rc;
    if ((rc = grow_device(h, &h->d_spl_io, &h->d_spl_io_cap, s_r + s_a + s_iv + s_c + s_o + s_g)) != ESP_OK)
        return rc;
    uint8_t *p = (uint8_t *)h->d_spl_io;
    esp_splice_read *d_reads = (esp_splice_read *)p;
    uint8_t *d_arena = p + s_r;
    esp_n_interval *d_iv = (esp_n_interval *)(p + s_r + s_a);
    esp_splice_cand *d_cands = (esp_splice_cand *)(p + s_r + s_a + s_iv);
    esp_splice_result *d_out = (esp_splice_result *)(p + s_r + s_a + s_iv + s_c);
    uint32_t *d_cig = (uint32_t *)(p + s_r + s_a + s_iv + s_c + s_o);
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(d_reads, reads, n_reads * sizeof(esp_splice_read), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(d_arena, read_arena, read_arena_bytes, cudaMemcpyHostToDevice, st));
    CK(h, cudaMemsetAsync(d_arena + read_arena_bytes, 0, 16, st));
    if (read_n_iv_count)
        CK(h, cudaMemcpyAsync(d_iv, read_n_iv, read_n_iv_count * sizeof(esp_n_interval),
                              cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(d_cands, cands, n_cands * sizeof(esp_splice_cand), cudaMemcpyHostToDevice, st));
    SpliceBufs B;
    rc = enqueue_splice(h, g, d_reads, n_reads, maxL, d_arena, read_arena_bytes,
                        read_n_iv_count ? d_iv : nullptr, read_n_iv_count, d_cands, n_cands, *sp,
                        K, d_out, d_cig, cigar_stride, st, false, 0, B);
    if (rc != ESP_OK) return rc;
    CK(h, cudaMemcpyAsync(out, d_out, n_reads * sizeof(esp_splice_result), cudaMemcpyDeviceToHost, st));
    if (cigar && cigar_stride)
        CK(h, cudaMemcpyAsync(cigar, d_cig, n_reads * (size_t)cigar_stride * 4, cudaMemcpyDeviceToHost, st));
    // DP cell census of the batch (outside the result path)
    CK(h, cudaMemsetAsync(B.cells, 0, sizeof(unsigned long long), st));
    CK(h, esp::launch_count_cells(B.dp_pairs, B.dp_out, n_cands * esp::SPL_SLOTS, 1, B.cells,
                                  h->num_sms, st));
    unsigned long long cells = 0;
    CK(h, cudaMemcpyAsync(&cells, B.cells, sizeof(cells), cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    h->last_cells = cells;
    return ESP_OK;
}

int esp_batch_splice_device(esp_handle *h, const esp_genome *g, const esp_splice_read *reads,
                            uint64_t n_reads, uint32_t max_read_len, const uint8_t *read_arena,
                            uint64_t read_arena_bytes, const esp_n_interval *read_n_iv,
                            uint64_t read_n_iv_count, const esp_splice_cand *cands,
                            uint64_t n_cands, const esp_splice_params *sp,
                            const esp_extend_params *params, esp_splice_result *out,
                            uint32_t *cigar, uint32_t cigar_stride, void *stream) {
    if (!h || !g || !sp || !params || !out || (n_reads && (!reads || !read_arena)) ||
        (n_cands && !cands))
        return fail(h, ESP_EINVAL, "null argument");
    if (max_read_len < 1 || max_read_len > 32767) return fail(h, ESP_EDOMAIN, "read length");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    CK(h, cudaSetDevice(h->device));
    SpliceBufs B;
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    return enqueue_splice(h, g, reads, n_reads, max_read_len, read_arena, read_arena_bytes,
                          read_n_iv_count ? read_n_iv : nullptr, read_n_iv_count, cands, n_cands,
                          *sp, K, out, cigar, cigar_stride, st, false, 0, B);
}

}  // extern "C"
