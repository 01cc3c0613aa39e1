// spliced.cu -- the spliced pseudo-reference DP of crates/map/src/splice.rs
// (align_spliced :617-664 after prepare_spliced :565-607; stitch_cigar
// :435-493; SplicedAlignment::genomic_start :414-424) over a resident genome.
//
// The caller supplies, per read, the exon slices prepare_spliced chose (the
// junction refinement and guards run upstream).  Three device stages on the
// handle's stream: (1) gather -- one thread per read packs its
// pseudo-reference (the concatenated slices, 2-bit) from the genome into a
// private, 16-byte-aligned stretch of a scratch arena; (2) the batched
// extend_hint DP against it along the read's hint diagonal (the direct
// diagonal for align_spliced; the intron-chain fast path passes its own
// per read, spliced_batch); (3) stitch -- one
// thread per read maps the pseudo-reference CIGAR back to the genome,
// inserting an intron of exons[i+1].start - exons[i].end at every seam, and
// the pseudo start back to a genomic start.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "esp_device.cuh"
#include "esp_host.h"

namespace {

using esp::load1;

struct SplicedDev {
    uint64_t pseudo_pos;  // base offset of the read's pseudo-reference (multiple of 64)
    uint32_t exon_first, exon_count, contig, pad;
};

__global__ void spliced_gather(const SplicedDev *__restrict__ R, uint64_t n,
                               const esp_exon *__restrict__ exons,
                               const esp_contig *__restrict__ contigs,
                               const uint8_t *__restrict__ g_arena, uint8_t *__restrict__ pseudo) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const SplicedDev d = R[r];
        const esp_contig C = contigs[d.contig];
        uint8_t *out = pseudo + (d.pseudo_pos >> 2);
        uint32_t acc = 0, k = 0;
        uint64_t w = 0;
        for (uint32_t e = 0; e < d.exon_count; e++) {
            const esp_exon x = exons[d.exon_first + e];
            for (uint32_t p = x.start; p < x.end; p++) {
                acc = (acc << 2) | load1(g_arena, C.base + p);
                if (++k == 4) {
                    out[w++] = (uint8_t)acc;
                    acc = 0;
                    k = 0;
                }
            }
        }
        if (k) out[w] = (uint8_t)(acc << (2 * (4 - k)));
    }
}

// extend.rs:254-282 push_op
struct OpSink {
    uint32_t *v;
    uint32_t n, cap;
    __device__ void push(uint32_t code, uint32_t len) {
        if (n > 0 && n <= cap && (v[n - 1] & 15u) == code) {
            v[n - 1] += len << 4;
            return;
        }
        if (n < cap) v[n] = (len << 4) | code;
        n++;
    }
};

__global__ void spliced_stitch(const SplicedDev *__restrict__ R, uint64_t n,
                               const esp_exon *__restrict__ exons,
                               const esp_extension *__restrict__ ext,
                               const uint32_t *__restrict__ ext_cigar, uint32_t *stitched,
                               uint32_t stride, esp_spliced_result *__restrict__ out) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const SplicedDev d = R[r];
        const esp_extension x = ext[r];
        esp_spliced_result res{};
        res.ext = x;
        res.status = x.status;
        if (x.status != ESP_OK) {
            out[r] = res;
            continue;
        }
        const esp_exon *ex = exons + d.exon_first;
        const uint32_t nb = d.exon_count;
        auto ps_of = [&](uint32_t e) {  // pseudo start of exon e
            uint64_t s = 0;
            for (uint32_t q = 0; q < e; q++) s += ex[q].end - ex[q].start;
            return s;
        };
        OpSink o{stitched + (uint64_t)r * stride, 0, stride};
        const uint32_t *ops = ext_cigar + (uint64_t)r * stride;
        uint64_t p = x.ref_start;
        uint32_t ei = 0;
        uint64_t e_ps = 0, e_end = ex[0].end - ex[0].start;  // pseudo [start, end) of exon ei
        while (ei + 1 < nb && p >= e_end) {
            ei++;
            e_ps = e_end;
            e_end = e_ps + (ex[ei].end - ex[ei].start);
        }
        for (uint32_t k = 0; k < x.n_ops; k++) {
            const uint32_t code = ops[k] & 15u, len = ops[k] >> 4;
            if (code == ESP_OP_I || code == ESP_OP_S || code == ESP_OP_N) {
                o.push(code, len);
                continue;
            }
            uint64_t remaining = len;
            while (remaining > 0) {
                if (ei >= nb) {
                    o.push(code, (uint32_t)remaining);
                    p += remaining;
                    break;
                }
                if (p < e_ps) p = e_ps;  // snap into the exon slice
                uint64_t in_exon = e_end > p ? e_end - p : 0;
                uint64_t take = remaining < in_exon ? remaining : in_exon;
                if (take) o.push(code, (uint32_t)take);
                p += take;
                remaining -= take;
                if (remaining > 0) {
                    if (ei + 1 >= nb) {
                        o.push(code, (uint32_t)remaining);
                        p += remaining;
                        break;
                    }
                    o.push(ESP_OP_N, ex[ei + 1].start - ex[ei].end);
                    ei++;
                    e_ps = e_end;
                    e_end = e_ps + (ex[ei].end - ex[ei].start);
                }
            }
        }
        // genomic_start: the pseudo start mapped back through the slices
        uint32_t gs = 0;
        bool found = false;
        uint64_t s = 0;
        for (uint32_t e = 0; e < nb && !found; e++) {
            uint64_t len = ex[e].end - ex[e].start;
            if (x.ref_start >= s && x.ref_start < s + len) {
                gs = ex[e].start + (uint32_t)(x.ref_start - s);
                found = true;
            }
            s += len;
        }
        if (!found) {
            uint64_t last = ps_of(nb - 1);
            gs = ex[nb - 1].start + (uint32_t)(x.ref_start > last ? x.ref_start - last : 0);
        }
        res.genomic_start = gs;
        res.n_ops = o.n;
        if (o.n > stride) res.status = ESP_ECAP;
        out[r] = res;
    }
}

}  // namespace

int spliced_batch(esp_handle *h, const esp_genome *g, const esp_spliced_read *reads, uint64_t n,
                  const uint8_t *read_arena, uint64_t read_arena_bytes,
                  const esp_n_interval *read_iv, uint64_t n_read_iv, const esp_exon *exons,
                  uint64_t n_exons, const esp_extend_params *params, const int64_t *hint_offset,
                  esp_spliced_result *out, uint32_t *ext_cigar, uint32_t *stitched_cigar,
                  uint32_t cigar_stride) {
    if (!h || !g || !params || (n && (!reads || !read_arena || !exons || !out || !ext_cigar ||
                                      !stitched_cigar)) ||
        (n_read_iv && !read_iv))
        return fail(h, ESP_EINVAL, "null argument");
    if (n == 0) return ESP_OK;
    if (cigar_stride == 0) return fail(h, ESP_EINVAL, "zero CIGAR stride");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    // host side: pseudo-reference placement, DP pairs and their N intervals
    std::vector<SplicedDev> dev(n);
    std::vector<esp_pair> pairs(n);
    std::vector<esp_n_interval> iv;
    uint64_t pseudo_bases = 0;
    uint32_t max_m = 1, max_w = 1;
    for (uint64_t r = 0; r < n; r++) {
        const esp_spliced_read &R = reads[r];
        if (R.contig >= g->contigs.size() || R.exon_count == 0 ||
            (uint64_t)R.exon_first + R.exon_count > n_exons ||
            R.read_pos + R.read_len > read_arena_bytes * 4 ||
            (uint64_t)R.n_first + R.n_read > n_read_iv)
            return fail(h, ESP_EINVAL, "read record outside its tables");
        const esp_contig &C = g->contigs[R.contig];
        uint64_t total = 0;
        for (uint32_t e = 0; e < R.exon_count; e++) {
            const esp_exon &x = exons[R.exon_first + e];
            if (x.end < x.start || x.end > C.len) return fail(h, ESP_EINVAL, "exon outside its contig");
            if (e && x.start < exons[R.exon_first + e - 1].end)
                return fail(h, ESP_EINVAL, "exons overlap or are out of order");
            total += x.end - x.start;
        }
        if (R.read_len > 32767 || total > 32767)
            return fail(h, ESP_EDOMAIN, "read or pseudo-reference longer than 32767");
        dev[r] = SplicedDev{pseudo_bases, R.exon_first, R.exon_count, R.contig, 0};
        esp_pair &P = pairs[r];
        P.read_pos = R.read_pos;
        P.read_len = R.read_len;
        P.win_pos = pseudo_bases;
        P.win_len = (uint32_t)total;
        const int64_t off = hint_offset ? hint_offset[r] : 0;
        if (off < -(1ll << 30) || off > (1ll << 30))
            return fail(h, ESP_EDOMAIN, "hint offset out of range");
        P.band_offset = (int32_t)off;
        P.band_half = 30;
        P.n_first = (uint32_t)iv.size();
        for (uint32_t q = 0; q < R.n_read; q++) iv.push_back(read_iv[R.n_first + q]);
        uint32_t nw = 0;
        uint64_t at = 0;  // pseudo offset of the current exon
        for (uint32_t e = 0; e < R.exon_count; e++) {  // genome N runs clipped per slice
            const esp_exon &x = exons[R.exon_first + e];
            for (uint32_t q = 0; q < C.n_count; q++) {
                const esp_n_interval &v = g->h_iv[C.n_first + q];
                uint32_t a = std::max(v.start, x.start), b = std::min(v.end, x.end);
                if (a < b) {
                    iv.push_back({(uint32_t)(at + a - x.start), (uint32_t)(at + b - x.start)});
                    nw++;
                }
            }
            at += x.end - x.start;
        }
        if (R.n_read > 65535 || nw > 65535) return fail(h, ESP_EDOMAIN, "too many N runs");
        P.n_read = (uint16_t)R.n_read;
        P.n_win = (uint16_t)nw;
        pseudo_bases += (total + 63) / 64 * 64;
        max_m = std::max(max_m, R.read_len);
        max_w = std::max(max_w, (uint32_t)total);
    }
    CK(h, cudaSetDevice(h->device));
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t pseudo_bytes = pseudo_bases / 4 + 16;
    size_t o_dev = 0, o_pairs = o_dev + al(n * sizeof(SplicedDev)),
           o_iv = o_pairs + al(n * sizeof(esp_pair)), o_ex = o_iv + al(iv.size() * 8 + 8),
           o_rd = o_ex + al(n_exons * sizeof(esp_exon)), o_ps = o_rd + al(read_arena_bytes + 16),
           o_ext = o_ps + al(pseudo_bytes), o_res = o_ext + al(n * sizeof(esp_extension)),
           o_ec = o_res + al(n * sizeof(esp_spliced_result)),
           o_sc = o_ec + al(n * (size_t)cigar_stride * 4),
           total_bytes = o_sc + al(n * (size_t)cigar_stride * 4);
    int rc;
    if ((rc = grow_device(h, &h->d_spl_io, &h->d_spl_io_cap, total_bytes)) != ESP_OK) return rc;
    uint8_t *b = (uint8_t *)h->d_spl_io;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(b + o_dev, dev.data(), n * sizeof(SplicedDev), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(b + o_pairs, pairs.data(), n * sizeof(esp_pair), cudaMemcpyHostToDevice, st));
    if (!iv.empty())
        CK(h, cudaMemcpyAsync(b + o_iv, iv.data(), iv.size() * 8, cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(b + o_ex, exons, n_exons * sizeof(esp_exon), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(b + o_rd, read_arena, read_arena_bytes, cudaMemcpyHostToDevice, st));
    CK(h, cudaMemsetAsync(b + o_rd + read_arena_bytes, 0, 16, st));
    CK(h, cudaMemsetAsync(b + o_ps, 0, pseudo_bytes, st));
    const int grid = (int)std::min<uint64_t>((n + 127) / 128, (uint64_t)h->num_sms * 8);
    spliced_gather<<<grid, 128, 0, st>>>((const SplicedDev *)(b + o_dev), n,
                                         (const esp_exon *)(b + o_ex), g->d_contigs, g->d_arena,
                                         b + o_ps);
    CK(h, cudaGetLastError());
    Limits L1, L2;
    add_limits(L1, max_m, max_w, 30);
    add_limits(L2, max_m, max_w, -1);
    rc = enqueue_batch(h, ESP_MODE_HINT, (const esp_pair *)(b + o_pairs), n, b + o_rd,
                       read_arena_bytes, (const esp_n_interval *)(b + o_iv), iv.size(), K, L1, L2,
                       (esp_extension *)(b + o_ext), (uint32_t *)(b + o_ec), cigar_stride, st,
                       b + o_ps, pseudo_bytes - 16);
    if (rc != ESP_OK) return rc;
    spliced_stitch<<<grid, 128, 0, st>>>((const SplicedDev *)(b + o_dev), n,
                                         (const esp_exon *)(b + o_ex),
                                         (const esp_extension *)(b + o_ext),
                                         (const uint32_t *)(b + o_ec), (uint32_t *)(b + o_sc),
                                         cigar_stride, (esp_spliced_result *)(b + o_res));
    CK(h, cudaGetLastError());
    CK(h, cudaMemcpyAsync(out, b + o_res, n * sizeof(esp_spliced_result), cudaMemcpyDeviceToHost, st));
    CK(h, cudaMemcpyAsync(ext_cigar, b + o_ec, n * (size_t)cigar_stride * 4, cudaMemcpyDeviceToHost, st));
    CK(h, cudaMemcpyAsync(stitched_cigar, b + o_sc, n * (size_t)cigar_stride * 4, cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    return ESP_OK;
}

extern "C" int esp_batch_spliced_host(esp_handle *h, const esp_genome *g,
                                      const esp_spliced_read *reads, uint64_t n,
                                      const uint8_t *read_arena, uint64_t read_arena_bytes,
                                      const esp_n_interval *read_iv, uint64_t n_read_iv,
                                      const esp_exon *exons, uint64_t n_exons,
                                      const esp_extend_params *params, esp_spliced_result *out,
                                      uint32_t *ext_cigar, uint32_t *stitched_cigar,
                                      uint32_t cigar_stride) {
    // align_spliced runs extend_hint along the direct diagonal (offset 0)
    return spliced_batch(h, g, reads, n, read_arena, read_arena_bytes, read_iv, n_read_iv, exons,
                         n_exons, params, nullptr, out, ext_cigar, stitched_cigar, cigar_stride);
}
