// splice.cu -- GB300 splice-rescue flank DP around the batched Gotoh kernel
// (crates/map/src/split.rs:150-321, :468-570; splice.rs:63-103, :324-340).
//
// A batch of reads, each with its library candidates in library order, runs
// in three stages on one stream:
//   1. splice_build (one thread per read): filter candidates as
//      channel_a_with_policy does (strand, intron length, NonCanonical with
//      support < 2), read the junction signal from the resident genome, and
//      expand every surviving candidate into its breakpoint retries: for each
//      dro in [max(ts-5,1), min(ts+5, L-1)] one DP pair for the left segment
//      read[..dro] against [j.start-(dro+30), j.start) and one for the right
//      segment read[dro..] against [j.end, j.end+(L-dro)+30) -- 22 slots per
//      candidate, unused slots are empty pairs;
//   2. the persistent Gotoh kernel in extend_hint mode over all slots (length
//      binned, so the many left/right geometries still run warp-uniform);
//   3. splice_select (one thread per read): the gates and totals of
//      retry_tail_start, the strict-> choice over breakpoints (lowest dro) and
//      candidates (first in library order), build_rescue_ext and
//      rescue_cigar_valid.
#include <cuda_runtime.h>

#include <cstdint>

#include "esp_device.cuh"
#include "esp_internal.h"

namespace esp {

constexpr int SPL_RADIUS = 5;  // split.rs:30 TAIL_RETRY_RADIUS
constexpr int SPL_MARGIN = 30; // split.rs:60 TAIL_MARGIN
constexpr int SPL_COST = 4;    // splice.rs:57 SPLIT_COST

__device__ __forceinline__ bool g_is_n(const SpliceJob &J, const esp_contig &C, uint32_t pos) {
    return genome_is_n(GenomeView{J.g_arena, J.g_iv}, C, pos);
}

__device__ __forceinline__ uint8_t g_base(const SpliceJob &J, const esp_contig &C, uint32_t pos) {
    return genome_ascii(GenomeView{J.g_arena, J.g_iv}, C, pos);
}

__device__ __forceinline__ void g_dinuc(const SpliceJob &J, const esp_contig &C, uint32_t p,
                                        bool donor, uint8_t out[2]) {
    genome_dinuc(GenomeView{J.g_arena, J.g_iv}, C, p, donor, out);
}

__device__ __forceinline__ int splice_signal_dev(const uint8_t d[2], const uint8_t a[2],
                                                 bool minus) {
    return splice_signal_of(d, a, minus);
}

__device__ __forceinline__ int signal_score_dev(int sig, const esp_splice_params &sp) {
    return signal_bonus(sig, sp);
}

struct Windows {
    uint32_t l_lo, l_hi, r_lo, r_hi;
    bool ok;
};

// split.rs:172-182 window geometry of breakpoint dro.
__device__ __forceinline__ Windows windows_of(const esp_junction &j, uint32_t clen, uint32_t dro,
                                              uint32_t L) {
    Windows w;
    uint32_t llen = dro, rlen = L - dro;
    w.l_hi = min(j.start, clen);
    w.l_lo = w.l_hi > llen + SPL_MARGIN ? w.l_hi - (llen + SPL_MARGIN) : 0u;
    w.r_lo = j.end;
    uint64_t rh = (uint64_t)w.r_lo + rlen + SPL_MARGIN;
    w.r_hi = (uint32_t)(rh < clen ? rh : clen);
    w.ok = !(w.l_hi <= w.l_lo || w.r_hi <= w.r_lo);
    return w;
}

__device__ __forceinline__ void dro_range(uint32_t ts, uint32_t L, uint32_t &lo, uint32_t &hi) {
    lo = ts > (uint32_t)SPL_RADIUS ? ts - SPL_RADIUS : 0u;  // saturating_sub(5).max(1)
    if (lo < 1) lo = 1;
    hi = ts + SPL_RADIUS;
    uint32_t lm1 = L > 0 ? L - 1 : 0;  // min(read_len.saturating_sub(1))
    if (hi > lm1) hi = lm1;
}

// Relative N intervals of read[a, b) (read list, relative to the read) into
// dst; returns count or -1 on overflow.
__device__ int clip_read_iv(const esp_n_interval *iv, uint32_t cnt, uint32_t a, uint32_t b,
                            esp_n_interval *dst, int cap) {
    int k = 0;
    for (uint32_t q = 0; q < cnt; q++) {
        uint32_t s = max(iv[q].start, a), e = min(iv[q].end, b);
        if (s < e) {
            if (k >= cap) return -1;
            dst[k].start = s - a;
            dst[k].end = e - a;
            k++;
        }
    }
    return k;
}

// Relative N intervals of contig window [a, b).
__device__ int clip_genome_iv(const SpliceJob &J, const esp_contig &C, uint32_t a, uint32_t b,
                              esp_n_interval *dst, int cap) {
    const esp_n_interval *iv = J.g_iv + C.n_first;
    uint32_t lo = 0, hi = C.n_count;
    while (lo < hi) {  // first interval ending after a
        uint32_t mid = (lo + hi) >> 1;
        if (iv[mid].end <= a) lo = mid + 1;
        else hi = mid;
    }
    int k = 0;
    for (uint32_t q = lo; q < C.n_count && iv[q].start < b; q++) {
        uint32_t s = max(iv[q].start, a), e = min(iv[q].end, b);
        if (s < e) {
            if (k >= cap) return -1;
            dst[k].start = s - a;
            dst[k].end = e - a;
            k++;
        }
    }
    return k;
}

__global__ void splice_build(SpliceJob J) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < J.n_reads;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const esp_splice_read R = J.reads[r];
        const uint32_t L = R.read_len;
        bool ctg_ok = R.contig < J.n_contigs;
        esp_contig C = ctg_ok ? J.contigs[R.contig] : esp_contig{};
        uint32_t lo_dro, hi_dro;
        dro_range(R.tail_start, L, lo_dro, hi_dro);
        int32_t read_status = ESP_OK;
        for (uint32_t c = 0; c < R.cand_count; c++) {
            uint64_t item = (uint64_t)R.cand_first + c;
            const esp_splice_cand cd = J.cands[item];
            const esp_junction &j = cd.j;
            SpliceItem it;
            it.valid = 0;
            it.signal = ESP_SIG_NONCANONICAL;
            // channel_a_with_policy filters (split.rs:508-521)
            bool ok = ctg_ok && j.contig == R.contig;
            if (J.retry_only) {
                it.signal = J.forced_signal;  // retry_tail_start takes the signal as given
            } else {
                if (ok && ((j.minus_strand != 0) != (R.minus != 0))) ok = false;
                uint32_t intron = j.end - j.start;
                if (ok && (intron < J.sp.min_intron || intron > J.sp.max_intron)) ok = false;
            }
            if (ok && !J.retry_only) {
                uint8_t d[2], a[2];
                g_dinuc(J, C, j.start, true, d);
                g_dinuc(J, C, j.end, false, a);
                it.signal = splice_signal_dev(d, a, j.minus_strand != 0);
                if (it.signal == ESP_SIG_NONCANONICAL && cd.support < 2) ok = false;
            }
            it.valid = ok ? 1 : 0;
            for (int s = 0; s < 2 * (2 * SPL_RADIUS + 1); s++) {
                uint64_t slot = item * SPL_SLOTS + (uint64_t)s;
                uint32_t dro = lo_dro + (uint32_t)(s >> 1);
                esp_pair P{};
                P.band_offset = 0;
                P.band_half = 30;
                Windows w{};
                if (ok && dro <= hi_dro) w = windows_of(j, C.len, dro, L);
                if (ok && dro <= hi_dro && w.ok) {
                    bool left = (s & 1) == 0;
                    uint32_t ga = left ? w.l_lo : w.r_lo, gb = left ? w.l_hi : w.r_hi;
                    P.read_pos = R.read_pos + (left ? 0 : dro);
                    P.read_len = left ? dro : L - dro;
                    P.win_pos = C.base + ga;
                    P.win_len = gb - ga;
                    if (J.dp_iv) {
                        esp_n_interval *dst = J.dp_iv + slot * SPL_IVCAP;
                        int nr = clip_read_iv(J.read_iv + R.n_first, R.n_read, left ? 0 : dro,
                                              left ? dro : L, dst, SPL_IVCAP);
                        int nw = nr < 0 ? -1
                                        : clip_genome_iv(J, C, ga, gb, dst + nr, SPL_IVCAP - nr);
                        if (nr < 0 || nw < 0) {
                            read_status = ESP_EDOMAIN;  // more N runs than a slot holds
                            P.read_len = 0;
                        } else {
                            P.n_first = (uint32_t)(slot * SPL_IVCAP);
                            P.n_read = (uint16_t)nr;
                            P.n_win = (uint16_t)nw;
                        }
                    }
                }
                J.dp_pairs[slot] = P;
            }
            J.items[item] = it;
        }
        J.read_status[r] = read_status;
    }
}

// cigar_ref_end (span.rs:29-38) of an extension CIGAR, truncated to u32.
__device__ __forceinline__ uint32_t ref_end_of(uint32_t pos, const uint32_t *ops, uint32_t n) {
    uint64_t r = pos;
    for (uint32_t k = 0; k < n; k++) {
        uint32_t c = ops[k] & 15u;
        if (c == ESP_OP_M || c == ESP_OP_D || c == ESP_OP_N) r += ops[k] >> 4;
    }
    return (uint32_t)r;
}

__global__ void splice_select(SpliceJob J) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < J.n_reads;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const esp_splice_read R = J.reads[r];
        const uint32_t L = R.read_len;
        esp_splice_result res;
        res.found = 0;
        res.cand = -1;
        res.dro = 0;
        res.pos = 0;
        res.score = 0;
        res.signal = 0;
        res.n_ops = 0;
        res.status = J.read_status[r];
        uint32_t *cig = J.cigar + r * (uint64_t)J.cigar_stride;
        if (res.status != ESP_OK || R.contig >= J.n_contigs) {
            if (res.status == ESP_OK) res.status = ESP_EINVAL;
            J.out[r] = res;
            continue;
        }
        const uint32_t clen = J.contigs[R.contig].len;
        uint32_t lo_dro, hi_dro;
        dro_range(R.tail_start, L, lo_dro, hi_dro);
        bool have = false;
        int best_c = -1;
        uint32_t best_dro = 0, best_lwin = 0;
        int32_t best_total = 0;
        uint64_t best_slot = 0;
        for (uint32_t c = 0; c < R.cand_count && res.status == ESP_OK; c++) {
            uint64_t item = (uint64_t)R.cand_first + c;
            const SpliceItem it = J.items[item];
            if (!it.valid) continue;
            const esp_splice_cand cd = J.cands[item];
            const int32_t sig_score = signal_score_dev(it.signal, J.sp);
            const int32_t lib_bonus = (int32_t)(min(cd.support, 10u) * 5u);
            // retry_tail_start (split.rs:165-221)
            bool rfound = false;
            int32_t rtotal = 0;
            uint32_t rdro = 0, rlwin = 0;
            uint64_t rslot = 0;
            for (uint32_t dro = lo_dro; dro <= hi_dro; dro++) {
                Windows w = windows_of(cd.j, clen, dro, L);
                if (!w.ok) continue;
                uint64_t slot = item * SPL_SLOTS + 2ull * (dro - lo_dro);
                const esp_extension le = J.dp_out[slot], re = J.dp_out[slot + 1];
                if (le.status != ESP_OK || re.status != ESP_OK) {
                    res.status = (le.status == ESP_ECAP || re.status == ESP_ECAP) ? ESP_ECAP
                                                                                 : ESP_EINVAL;
                    break;
                }
                uint32_t llen = dro, rlen = L - dro;
                uint64_t l_al = le.read_end > le.read_start ? le.read_end - le.read_start : 0;
                uint64_t r_al = re.read_end > re.read_start ? re.read_end - re.read_start : 0;
                if (l_al * 5 < (uint64_t)llen * 4 || r_al * 5 < (uint64_t)rlen * 4) continue;
                if (le.read_end != llen || re.read_start != 0 || re.ref_start != 0) continue;
                const uint32_t *lops = J.dp_cig + slot * (uint64_t)J.dp_stride;
                if (ref_end_of(w.l_lo + le.ref_start, lops, le.n_ops) != cd.j.start) continue;
                int32_t total = le.score + re.score + sig_score + lib_bonus - SPL_COST;
                if (!rfound || total > rtotal) {
                    rfound = true;
                    rtotal = total;
                    rdro = dro;
                    rlwin = w.l_lo;
                    rslot = slot;
                }
            }
            if (res.status != ESP_OK) break;
            if (J.item_out) {
                SpliceItemOut io;
                io.found = rfound ? 1 : 0;
                io.dro = rdro;
                io.left_win_lo = rlwin;
                io.total = rtotal;
                io.slot = rslot;
                J.item_out[item] = io;
            }
            if (rfound && (!have || rtotal > best_total)) {  // ties keep the first candidate
                have = true;
                best_c = (int)c;
                best_total = rtotal;
                best_dro = rdro;
                best_lwin = rlwin;
                best_slot = rslot;
            }
        }
        if (res.status == ESP_OK && have) {
            // build_rescue_ext: left.cigar + N(intron) + right.cigar (push_op)
            const esp_splice_cand cd = J.cands[(uint64_t)R.cand_first + best_c];
            const esp_extension le = J.dp_out[best_slot], re = J.dp_out[best_slot + 1];
            const uint32_t *lops = J.dp_cig + best_slot * (uint64_t)J.dp_stride;
            const uint32_t *rops = J.dp_cig + (best_slot + 1) * (uint64_t)J.dp_stride;
            uint32_t n = 0;
            bool over = false;
            int prev = -1;
            auto push = [&](uint32_t op, uint32_t len) {
                if ((int)op == prev) {
                    cig[n - 1] += len << 4;
                } else if (n < J.cigar_stride) {
                    cig[n++] = (len << 4) | op;
                    prev = (int)op;
                } else {
                    over = true;
                }
            };
            for (uint32_t k = 0; k < le.n_ops; k++) push(lops[k] & 15u, lops[k] >> 4);
            push(ESP_OP_N, cd.j.end - cd.j.start);
            for (uint32_t k = 0; k < re.n_ops; k++) push(rops[k] & 15u, rops[k] >> 4);
            uint32_t pos = best_lwin + le.ref_start;
            if (over) {
                res.status = ESP_ECAP;
            } else {
                // rescue_cigar_valid (split.rs:282-321) with cigar_conserving
                uint64_t total_q = 0, refp = pos;
                bool valid = true, found_j = false;
                for (uint32_t k = 0; k < n; k++) {
                    uint32_t op = cig[k] & 15u, len = cig[k] >> 4;
                    if (op == ESP_OP_M || op == ESP_OP_I || op == ESP_OP_S) total_q += len;
                }
                if (total_q != L) valid = false;
                for (uint32_t k = 0; k < n && valid; k++) {
                    uint32_t op = cig[k] & 15u, len = cig[k] >> 4;
                    if (len == 0) valid = false;
                    else if (op == ESP_OP_S && k != 0 && k + 1 != n) valid = false;
                    else if (op == ESP_OP_N) {
                        if (k == 0 || k + 1 == n) valid = false;
                        else {
                            if (refp == cd.j.start && refp + len == cd.j.end) found_j = true;
                            refp += len;
                        }
                    } else if (op == ESP_OP_M || op == ESP_OP_D) {
                        refp += len;
                    }
                }
                if (valid && found_j && refp <= 0xffffffffull) {
                    res.found = 1;
                    res.cand = best_c;
                    res.dro = best_dro;
                    res.pos = pos;
                    res.score = best_total;
                    res.signal = J.items[(uint64_t)R.cand_first + best_c].signal;
                    res.n_ops = n;
                }
            }
        }
        J.out[r] = res;
    }
}

cudaError_t launch_splice_build(const SpliceJob &J, int num_sms, cudaStream_t st) {
    if (J.n_reads == 0) return cudaSuccess;
    uint64_t need = (J.n_reads + 127) / 128;
    int grid = (int)(need < (uint64_t)num_sms * 8 ? need : (uint64_t)num_sms * 8);
    splice_build<<<grid, 128, 0, st>>>(J);
    return cudaGetLastError();
}

cudaError_t launch_splice_select(const SpliceJob &J, int num_sms, cudaStream_t st) {
    if (J.n_reads == 0) return cudaSuccess;
    uint64_t need = (J.n_reads + 127) / 128;
    int grid = (int)(need < (uint64_t)num_sms * 8 ? need : (uint64_t)num_sms * 8);
    splice_select<<<grid, 128, 0, st>>>(J);
    return cudaGetLastError();
}

}  // namespace esp
