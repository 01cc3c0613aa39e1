// esp_device.cuh -- device-side helpers shared by the GB300 kernels:
// 2-bit arena loads, N-interval masks, bounded spin helpers.
#pragma once

#include <cstdint>

#include "esperanto_gb300.h"

namespace esp {

// Load 16 consecutive bases starting at base position `p` of a 2-bit packed
// MSB-first arena (crates/map/src/fasta.rs:1-5 layout).  Result: base p in
// bits 31:30, p+1 in 29:28, ...  The arena is 4-byte aligned and padded by
// at least 8 bytes past its last base, so the two word loads stay in bounds.
__device__ __forceinline__ uint32_t load16(const uint8_t *__restrict__ arena, uint64_t p) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(arena);
    uint64_t bit = p * 2;                 // bit offset from arena start (big-endian view)
    uint64_t wi = bit >> 5;
    uint32_t sh = (uint32_t)(bit & 31);
    uint32_t a = __byte_perm(__ldg(w + wi), 0, 0x0123);
    uint32_t b = __byte_perm(__ldg(w + wi + 1), 0, 0x0123);
    return __funnelshift_l(b, a, sh);
}

// 2-bit code of one base.
__device__ __forceinline__ uint32_t load1(const uint8_t *__restrict__ arena, uint64_t p) {
    uint8_t byte = __ldg(arena + (p >> 2));
    return (byte >> (6 - 2 * (uint32_t)(p & 3))) & 3u;
}

// N-interval mask for 16 positions [q, q+16) of a sequence whose intervals
// (relative to the sequence start) are iv[0..cnt).  Bit 31-k set when
// position q+k is N (MSB-first, aligned with load16's layout).
__device__ __forceinline__ uint32_t nmask16(const esp_n_interval *__restrict__ iv, uint32_t cnt,
                                            int64_t q) {
    uint32_t m = 0;
    for (uint32_t k = 0; k < cnt; k++) {
        int64_t s = iv[k].start, e = iv[k].end;
        int64_t a = s > q ? s : q;
        int64_t b = e < q + 16 ? e : q + 16;
        if (a < b) {
            // bits for positions [a, b): MSB-first => bit (31 - (pos - q))
            uint32_t len = (uint32_t)(b - a), off = (uint32_t)(a - q);
            uint32_t run = (len >= 32) ? 0xffffffffu : ((1u << len) - 1u);
            m |= (run << (32 - len)) >> off;
        }
    }
    return m;
}

// Is position q of a sequence inside one of its N intervals?
__device__ __forceinline__ bool is_n(const esp_n_interval *__restrict__ iv, uint32_t cnt,
                                     int64_t q) {
    for (uint32_t k = 0; k < cnt; k++)
        if (q >= (int64_t)iv[k].start && q < (int64_t)iv[k].end) return true;
    return false;
}

// Base code (0..3, 4 = N) of position q of a sequence.
__device__ __forceinline__ uint32_t code5(const uint8_t *__restrict__ arena, uint64_t pos,
                                          const esp_n_interval *__restrict__ iv, uint32_t cnt,
                                          int64_t q) {
    if (cnt && is_n(iv, cnt, q)) return 4;
    return load1(arena, pos + (uint64_t)q);
}

// A resident genome as kernels see it: the 2-bit arena and the merged N
// intervals of every contig (contig C owns iv[C.n_first, C.n_first + C.n_count)).
struct GenomeView {
    const uint8_t *arena;
    const esp_n_interval *iv;
};

// fasta.rs:117-134: binary search over the contig's merged N intervals.
__device__ __forceinline__ bool genome_is_n(const GenomeView &G, const esp_contig &C,
                                            uint32_t pos) {
    uint32_t lo = 0, hi = C.n_count;
    const esp_n_interval *iv = G.iv + C.n_first;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (pos < iv[mid].start) hi = mid;
        else if (pos >= iv[mid].end) lo = mid + 1;
        else return true;
    }
    return false;
}

// Base code (0..3, 4 = N) of contig position pos (fasta.rs:105-116 base).
__device__ __forceinline__ uint32_t genome_code(const GenomeView &G, const esp_contig &C,
                                                uint32_t pos) {
    return genome_is_n(G, C, pos) ? 4u : load1(G.arena, C.base + pos);
}

// ASCII base of contig position pos (base + to_ascii).
__device__ __forceinline__ uint8_t genome_ascii(const GenomeView &G, const esp_contig &C,
                                                uint32_t pos) {
    const uint8_t B[5] = {'A', 'C', 'G', 'T', 'N'};
    return B[genome_code(G, C, pos)];
}

// splice.rs:324-340 dinuc (donor at p, acceptor ending at p; N-padded)
__device__ __forceinline__ void genome_dinuc(const GenomeView &G, const esp_contig &C, uint32_t p,
                                             bool donor, uint8_t out[2]) {
    out[0] = out[1] = 'N';
    if (!donor && p < 2) return;
    uint32_t a = donor ? p : p - 2, b = donor ? p + 2 : p;
    if (a >= C.len) return;
    if (b > C.len) b = C.len;
    for (uint32_t q = a; q < b; q++) out[q - a] = genome_ascii(G, C, q);
}

// splice.rs:78-103 splice_signal (inputs are uppercase here)
__device__ __forceinline__ int splice_signal_of(const uint8_t d[2], const uint8_t a[2],
                                                bool minus) {
    auto is = [](const uint8_t x[2], char c0, char c1) { return x[0] == c0 && x[1] == c1; };
    if (!minus) {
        if (is(d, 'G', 'T') && is(a, 'A', 'G')) return ESP_SIG_GTAG;
        if (is(d, 'G', 'C') && is(a, 'A', 'G')) return ESP_SIG_GCAG;
        if (is(d, 'A', 'T') && is(a, 'A', 'C')) return ESP_SIG_ATAC;
        return ESP_SIG_NONCANONICAL;
    }
    if (is(d, 'C', 'T') && is(a, 'A', 'C')) return ESP_SIG_GTAG;
    if (is(d, 'C', 'T') && is(a, 'G', 'C')) return ESP_SIG_GCAG;
    if (is(d, 'G', 'T') && is(a, 'A', 'T')) return ESP_SIG_ATAC;
    return ESP_SIG_NONCANONICAL;
}

// splice.rs:63-71 SpliceSignal::score
__device__ __forceinline__ int signal_bonus(int sig, const esp_splice_params &sp) {
    switch (sig) {
    case ESP_SIG_GTAG: return sp.gt_ag_bonus;
    case ESP_SIG_GCAG: return sp.gc_ag_bonus;
    case ESP_SIG_ATAC: return sp.at_ac_bonus;
    default: return -sp.noncanonical_penalty;
    }
}

// PTX prmt in its default mode: selector nibble bit 3 replicates the sign of
// the selected byte, so a selector of c*0x1111 + 0x8880 returns byte c of
// {hi:lo} sign-extended to 32 bits.
__device__ __forceinline__ int32_t prmt_sx(uint32_t lo, uint32_t hi, uint32_t sel) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(sel));
    return (int32_t)r;
}

}  // namespace esp
