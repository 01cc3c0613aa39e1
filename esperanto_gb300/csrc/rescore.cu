// rescore.cu -- strict rescoring of placements on GB300
// (crates/map/src/align.rs:1060-1165 Aligner::rescore_with).
//
// One thread per placement walks its CIGAR against the resident genome:
// M columns score match / mismatch (an N on either side is neither scored
// nor counted; the editing direction exempts its substitution from the
// mismatch charge but still counts it), I/D charge open + n*ext, S counts
// clipped bases, N (intron) adds the known-junction bonus when the library
// holds (contig, start, end) on either strand, else the better of the two
// strands' motif scores minus the intron-length penalty.  Genome bases are
// read in place (2-bit + N runs); the N runs of a contig are walked with a
// cursor inside each M run instead of a search per base.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "esp_device.cuh"
#include "esp_host.h"

namespace {

using esp::load1;

constexpr int kPenaltyTab = 64;

// splice.rs:119-121 intron_length_penalty = (8 |log10(max(len,1)) - 3|) as
// i32, as integer thresholds: up[k-1] = least len >= 1000 whose penalty is
// >= k, lo[k-1] = greatest len <= 1000 whose penalty is >= k.  Found by
// bisection over the host's own f64 evaluation, so the device reproduces
// the host's result for every u32 length, exact powers of ten included.
struct PenaltyTab {
    uint32_t up[kPenaltyTab], lo[kPenaltyTab];
    int n_up, n_lo;
};

int32_t host_penalty(uint32_t len) {
    double x = (double)(len > 1 ? len : 1);
    return (int32_t)(8.0 * std::fabs(std::log10(x) - 3.0));
}

const PenaltyTab &penalty_tab() {
    static PenaltyTab T;
    static std::once_flag once;
    std::call_once(once, [] {
        T.n_up = T.n_lo = 0;
        for (int k = 1; k <= kPenaltyTab; k++) {
            if (host_penalty(0xffffffffu) >= k) {  // nondecreasing on [1000, 2^32)
                uint64_t a = 1000, b = 0xffffffffull;
                while (a < b) {
                    uint64_t mid = (a + b) / 2;
                    if (host_penalty((uint32_t)mid) >= k) b = mid;
                    else a = mid + 1;
                }
                T.up[T.n_up++] = (uint32_t)a;
            }
            if (host_penalty(1) >= k) {  // nonincreasing on [1, 1000]
                uint32_t a = 1, b = 1000;
                while (a < b) {
                    uint32_t mid = (a + b + 1) / 2;
                    if (host_penalty(mid) >= k) a = mid;
                    else b = mid - 1;
                }
                T.lo[T.n_lo++] = a;
            }
        }
    });
    return T;
}

struct RescoreJob {
    const esp_rescore_item *items;
    uint64_t n;
    const uint8_t *queries;
    uint64_t query_bytes;
    const uint32_t *ops;
    uint64_t n_ops;
    const esp_junction *lib;
    uint64_t n_lib;
    const uint8_t *g_arena;
    const esp_contig *contigs;
    uint32_t n_contigs;
    const esp_n_interval *g_iv;
    esp_strict_score *out;
    int32_t match, mismatch, gap_open, gap_ext;
    int32_t sig[4];   // motif scores GT-AG, GC-AG, AT-AC, non-canonical
    int32_t known_bonus;
    PenaltyTab pen;
};

__host__ __device__ int32_t penalty(const PenaltyTab &T, uint32_t len) {
    int k = 0;
    if (len >= 1000) {
        while (k < T.n_up && T.up[k] <= len) k++;
    } else {
        while (k < T.n_lo && T.lo[k] >= len) k++;
    }
    return k;
}

// contig base as ASCII ('N' in an N run or past the end), one-off lookups
__device__ uint8_t base_at(const RescoreJob &J, const esp_contig &C, uint32_t i) {
    if (i >= C.len) return 'N';
    const esp_n_interval *iv = J.g_iv + C.n_first;
    uint32_t lo = 0, hi = C.n_count;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (iv[mid].end <= i) lo = mid + 1;
        else hi = mid;
    }
    if (lo < C.n_count && iv[lo].start <= i) return 'N';
    const uint8_t B[4] = {'A', 'C', 'G', 'T'};
    return B[load1(J.g_arena, C.base + i)];
}

// splice.rs:78-103 splice_signal -> index into sig[] (bases already upper case)
__device__ int signal_of(uint8_t d0, uint8_t d1, uint8_t a0, uint8_t a1, bool minus) {
    if (!minus) {
        if (d0 == 'G' && d1 == 'T' && a0 == 'A' && a1 == 'G') return 0;
        if (d0 == 'G' && d1 == 'C' && a0 == 'A' && a1 == 'G') return 1;
        if (d0 == 'A' && d1 == 'T' && a0 == 'A' && a1 == 'C') return 2;
        return 3;
    }
    if (d0 == 'C' && d1 == 'T' && a0 == 'A' && a1 == 'C') return 0;
    if (d0 == 'C' && d1 == 'T' && a0 == 'G' && a1 == 'C') return 1;
    if (d0 == 'G' && d1 == 'T' && a0 == 'A' && a1 == 'T') return 2;
    return 3;
}

__device__ bool lib_contains(const RescoreJob &J, uint32_t contig, uint32_t start, uint32_t end) {
    uint64_t lo = 0, hi = J.n_lib;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        const esp_junction &j = J.lib[mid];
        if (j.contig == contig && j.start == start && j.end == end) return true;
        bool less = j.contig < contig ||
                    (j.contig == contig && (j.start < start || (j.start == start && j.end < end)));
        if (less) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

__global__ void __launch_bounds__(128) rescore_kernel(RescoreJob J) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < J.n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const esp_rescore_item it = J.items[k];
        esp_strict_score s{};
        if (it.contig >= J.n_contigs || (uint64_t)it.op_first + it.op_count > J.n_ops ||
            it.query_pos + it.query_len > J.query_bytes) {
            s.status = ESP_EINVAL;
            J.out[k] = s;
            continue;
        }
        const esp_contig C = J.contigs[it.contig];
        const esp_n_interval *civ = J.g_iv + C.n_first;
        const uint8_t *q = J.queries + it.query_pos;
        int32_t score = 0;
        uint32_t ro = 0, rf = it.pos;
        for (uint32_t o = 0; o < it.op_count; o++) {
            const uint32_t op = J.ops[it.op_first + o];
            const uint32_t n = op >> 4, code = op & 15u;
            if (code == ESP_OP_M) {
                uint32_t avail = C.len > rf ? C.len - rf : 0;
                if (avail > n) avail = n;
                // first N run ending after rf; advanced with the position
                uint32_t a = 0, b = C.n_count;
                while (a < b) {
                    uint32_t mid = (a + b) >> 1;
                    if (civ[mid].end <= rf) a = mid + 1;
                    else b = mid;
                }
                for (uint32_t c = 0; c < n; c++) {
                    uint8_t qb = (uint64_t)ro + c < it.query_len ? q[ro + c] : (uint8_t)'N';
                    uint8_t rb = 'N';
                    if (c < avail) {
                        uint32_t g = rf + c;
                        while (a < C.n_count && civ[a].end <= g) a++;
                        if (!(a < C.n_count && civ[a].start <= g)) {
                            const uint8_t B[4] = {'A', 'C', 'G', 'T'};
                            rb = B[load1(J.g_arena, C.base + g)];
                        }
                    }
                    if (qb == 'N' || rb == 'N') continue;  // 0 score, uncounted
                    s.aligned++;
                    if (qb == rb) {
                        score += J.match;
                        s.matches++;
                    } else {
                        // extend.rs:87-93 exempt_dir; EditDir::exempt (:71-76)
                        int ed = (rb == 'A' && qb == 'G') ? 1 : ((rb == 'T' && qb == 'C') ? 0 : -1);
                        bool exempt = (it.edit_dir == ESP_EDIT_AG && ed == 1) ||
                                      (it.edit_dir == ESP_EDIT_TC && ed == 0);
                        if (!exempt) score += J.mismatch;
                        if (ed == 1) s.ea_ag++;
                        else if (ed == 0) s.ea_tc++;
                        else s.mm++;
                    }
                }
                ro += n;
                rf += n;
            } else if (code == ESP_OP_I) {
                score -= J.gap_open + J.gap_ext * (int32_t)n;
                s.aligned += n;
                s.ins++;
                ro += n;
            } else if (code == ESP_OP_D) {
                score -= J.gap_open + J.gap_ext * (int32_t)n;
                s.aligned += n;
                s.del++;
                rf += n;
            } else if (code == ESP_OP_S) {
                s.clipped += n;
                ro += n;
            } else {  // ESP_OP_N: intron
                const int32_t before = score;
                if (lib_contains(J, it.contig, rf, rf + n)) {
                    score += J.known_bonus;
                } else {
                    uint32_t r1 = rf == 0xffffffffu ? rf : rf + 1;
                    uint32_t n2 = n >= 2 ? n - 2 : 0, n1 = n >= 1 ? n - 1 : 0;
                    uint8_t d0 = base_at(J, C, rf), d1 = base_at(J, C, r1);
                    uint8_t a0 = base_at(J, C, rf + n2), a1 = base_at(J, C, rf + n1);
                    int32_t x = J.sig[signal_of(d0, d1, a0, a1, false)];
                    int32_t y = J.sig[signal_of(d0, d1, a0, a1, true)];
                    score += (x > y ? x : y) - penalty(J.pen, n);
                }
                s.n_splice++;
                s.splice_score += score - before;
                rf += n;
            }
        }
        s.score = score;
        s.status = ESP_OK;
        J.out[k] = s;
    }
}

}  // namespace

extern "C" {

int32_t esp_intron_length_penalty(uint32_t len) { return penalty(penalty_tab(), len); }

int esp_batch_rescore_device(esp_handle *h, const esp_genome *g, const esp_rescore_item *items,
                             uint64_t n, const uint8_t *queries, uint64_t query_bytes,
                             const uint32_t *ops, uint64_t n_ops, const esp_junction *lib,
                             uint64_t n_lib, const esp_extend_params *params,
                             const esp_splice_params *sp, esp_strict_score *out, void *stream) {
    if (!h || !g || !params || (n && (!items || !out)) || (n_lib && !lib))
        return fail(h, ESP_EINVAL, "null argument");
    if (n == 0) return ESP_OK;
    CK(h, cudaSetDevice(h->device));
    RescoreJob J{};
    J.items = items;
    J.n = n;
    J.queries = queries;
    J.query_bytes = queries ? query_bytes : 0;
    J.ops = ops;
    J.n_ops = ops ? n_ops : 0;
    J.lib = lib;
    J.n_lib = n_lib;
    J.g_arena = g->d_arena;
    J.contigs = g->d_contigs;
    J.n_contigs = (uint32_t)g->contigs.size();
    J.g_iv = g->d_iv;
    J.out = out;
    J.match = params->match_score;
    J.mismatch = params->mismatch;
    J.gap_open = params->gap_open;
    J.gap_ext = params->gap_ext;
    // rescore_with uses SpliceParams::default() (align.rs:1062); sp overrides
    esp_splice_params d{20, 1000000, 4, 2, 1, 8, 6, 12};
    const esp_splice_params &P = sp ? *sp : d;
    J.sig[0] = P.gt_ag_bonus;
    J.sig[1] = P.gc_ag_bonus;
    J.sig[2] = P.at_ac_bonus;
    J.sig[3] = -P.noncanonical_penalty;
    J.known_bonus = P.known_bonus;
    J.pen = penalty_tab();
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    uint64_t need = (n + 127) / 128;
    int grid = (int)(need < (uint64_t)h->num_sms * 16 ? need : (uint64_t)h->num_sms * 16);
    rescore_kernel<<<grid, 128, 0, st>>>(J);
    CK(h, cudaGetLastError());
    h->launches = 1;
    return ESP_OK;
}

int esp_batch_rescore_host(esp_handle *h, const esp_genome *g, const esp_rescore_item *items,
                           uint64_t n, const uint8_t *queries, uint64_t query_bytes,
                           const uint32_t *ops, uint64_t n_ops, const esp_junction *lib,
                           uint64_t n_lib, const esp_extend_params *params,
                           const esp_splice_params *sp, esp_strict_score *out) {
    if (!h || !g || !params || (n && (!items || !out)) || (n_lib && !lib))
        return fail(h, ESP_EINVAL, "null argument");
    if (n == 0) return ESP_OK;
    CK(h, cudaSetDevice(h->device));
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    size_t o_items = 0, o_q = o_items + al(n * sizeof(esp_rescore_item)),
           o_ops = o_q + al(query_bytes + 1), o_lib = o_ops + al(n_ops * 4 + 4),
           o_out = o_lib + al(n_lib * sizeof(esp_junction) + 1),
           total = o_out + al(n * sizeof(esp_strict_score));
    int rc;
    if ((rc = grow_device(h, &h->d_bat, &h->d_bat_cap, total)) != ESP_OK) return rc;
    uint8_t *b = (uint8_t *)h->d_bat;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(b + o_items, items, n * sizeof(esp_rescore_item), cudaMemcpyHostToDevice, st));
    if (query_bytes) CK(h, cudaMemcpyAsync(b + o_q, queries, query_bytes, cudaMemcpyHostToDevice, st));
    if (n_ops) CK(h, cudaMemcpyAsync(b + o_ops, ops, n_ops * 4, cudaMemcpyHostToDevice, st));
    if (n_lib) CK(h, cudaMemcpyAsync(b + o_lib, lib, n_lib * sizeof(esp_junction), cudaMemcpyHostToDevice, st));
    rc = esp_batch_rescore_device(h, g, (const esp_rescore_item *)(b + o_items), n, b + o_q,
                                  query_bytes, (const uint32_t *)(b + o_ops), n_ops,
                                  (const esp_junction *)(b + o_lib), n_lib, params, sp,
                                  (esp_strict_score *)(b + o_out), st);
    if (rc != ESP_OK) return rc;
    CK(h, cudaMemcpyAsync(out, b + o_out, n * sizeof(esp_strict_score), cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    return ESP_OK;
}

}  // extern "C"
