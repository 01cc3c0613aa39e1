// myers.cu -- GB300 editing-aware bit-parallel Myers filters
// (crates/map/src/myers_ea.rs and crates/engine/src/myers.rs).
//
// One thread owns one read x text pair.  The pattern (m <= 256 bases) is a
// bit-vector of NW 32-bit limbs held in registers; the pattern-equality
// table Peq[text code][limb] lives in shared memory with a thread-private
// column per lane (conflict-free: limb w of code c of thread t is at
// ((c * NW + w) * blockDim + t)).  Each text column advances the whole
// bit-vector as one wide word: the match-propagation addition ripples its
// carry across limbs in a single add.cc/addc chain and the horizontal deltas
// shift across limbs through funnel shifts.  This is the ripple-carry form of
// engine/src/myers.rs:179-208; the edlib block form of myers_ea.rs:64-91
// computes the same column scores, so one kernel serves both.
//
// EA equality (myers_ea.rs:28-56, engine/src/myers.rs:111-123): read A
// matches text {A}, C matches {C,T}, G matches {G,A}, T matches {T}; a read
// or text base that is not A/C/G/T matches nothing.
#include <cuda_runtime.h>

#include <cstdint>

#include "esp_device.cuh"
#include "esp_internal.h"

namespace esp {

// sum[k] = a[k] + b[k] + carry over k = 0..NW-1 in one PTX carry chain.
template <int NW>
__device__ __forceinline__ void add_chain(uint32_t (&s)[NW], const uint32_t (&a)[NW],
                                          const uint32_t (&b)[NW]);

template <>
__device__ __forceinline__ void add_chain<1>(uint32_t (&s)[1], const uint32_t (&a)[1],
                                             const uint32_t (&b)[1]) {
    s[0] = a[0] + b[0];
}
template <>
__device__ __forceinline__ void add_chain<2>(uint32_t (&s)[2], const uint32_t (&a)[2],
                                             const uint32_t (&b)[2]) {
    asm("add.cc.u32 %0, %2, %4;\n\taddc.u32 %1, %3, %5;"
        : "=r"(s[0]), "=r"(s[1])
        : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
}
template <>
__device__ __forceinline__ void add_chain<3>(uint32_t (&s)[3], const uint32_t (&a)[3],
                                             const uint32_t (&b)[3]) {
    asm("add.cc.u32 %0, %3, %6;\n\taddc.cc.u32 %1, %4, %7;\n\taddc.u32 %2, %5, %8;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
}
template <>
__device__ __forceinline__ void add_chain<4>(uint32_t (&s)[4], const uint32_t (&a)[4],
                                             const uint32_t (&b)[4]) {
    asm("add.cc.u32 %0, %4, %8;\n\taddc.cc.u32 %1, %5, %9;\n\taddc.cc.u32 %2, %6, %10;\n\t"
        "addc.u32 %3, %7, %11;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]),
          "r"(b[3]));
}
template <>
__device__ __forceinline__ void add_chain<5>(uint32_t (&s)[5], const uint32_t (&a)[5],
                                             const uint32_t (&b)[5]) {
    asm("add.cc.u32 %0, %5, %10;\n\taddc.cc.u32 %1, %6, %11;\n\taddc.cc.u32 %2, %7, %12;\n\t"
        "addc.cc.u32 %3, %8, %13;\n\taddc.u32 %4, %9, %14;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(b[0]), "r"(b[1]),
          "r"(b[2]), "r"(b[3]), "r"(b[4]));
}
template <>
__device__ __forceinline__ void add_chain<6>(uint32_t (&s)[6], const uint32_t (&a)[6],
                                             const uint32_t (&b)[6]) {
    asm("add.cc.u32 %0, %6, %12;\n\taddc.cc.u32 %1, %7, %13;\n\taddc.cc.u32 %2, %8, %14;\n\t"
        "addc.cc.u32 %3, %9, %15;\n\taddc.cc.u32 %4, %10, %16;\n\taddc.u32 %5, %11, %17;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(b[0]),
          "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
}
template <>
__device__ __forceinline__ void add_chain<7>(uint32_t (&s)[7], const uint32_t (&a)[7],
                                             const uint32_t (&b)[7]) {
    asm("add.cc.u32 %0, %7, %14;\n\taddc.cc.u32 %1, %8, %15;\n\taddc.cc.u32 %2, %9, %16;\n\t"
        "addc.cc.u32 %3, %10, %17;\n\taddc.cc.u32 %4, %11, %18;\n\taddc.cc.u32 %5, %12, %19;\n\t"
        "addc.u32 %6, %13, %20;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]),
          "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]));
}
template <>
__device__ __forceinline__ void add_chain<8>(uint32_t (&s)[8], const uint32_t (&a)[8],
                                             const uint32_t (&b)[8]) {
    asm("add.cc.u32 %0, %8, %16;\n\taddc.cc.u32 %1, %9, %17;\n\taddc.cc.u32 %2, %10, %18;\n\t"
        "addc.cc.u32 %3, %11, %19;\n\taddc.cc.u32 %4, %12, %20;\n\taddc.cc.u32 %5, %13, %21;\n\t"
        "addc.cc.u32 %6, %14, %22;\n\taddc.u32 %7, %15, %23;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]),
          "=r"(s[7])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]),
          "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]),
          "r"(b[6]), "r"(b[7]));
}

constexpr int MY_BLOCK = 128;

// One pair.  flags: MYF_REVERSE (best start: read and text both reversed,
// myers_ea.rs:158-185), MYF_GLOBAL (engine global: leading column +1 per text
// base, engine/src/myers.rs:151-169).
template <int NW>
__device__ void myers_pair(const MyersJob &job, uint32_t k, uint32_t *__restrict__ peq) {
    const esp_myers_pair P = job.pairs[k];
    const int m = (int)P.read_len;
    const int64_t n = P.text_len;
    const bool rev = job.flags & MYF_REVERSE;
    const bool glob = job.flags & MYF_GLOBAL;
    esp_myers_result res;
    res.dist = m;
    res.pos = 0;
    res.status = ESP_OK;
    if (m == 0 || m > NW * 32) {
        job.out[k] = res;  // the host routed m = 0 / m > 256 before launch
        if (m > NW * 32) job.out[k].status = ESP_EINVAL;
        return;
    }
    const esp_n_interval *iv = job.n_iv + P.n_first;
    const uint32_t bs = blockDim.x, t = threadIdx.x;
    // Peq rows: text code 0..3, row 4 (text N) all zero.  Each 32-position
    // limb is built in registers: the 2-bit codes are split into a high-bit
    // and a low-bit mask (position k -> bit k) and combined per EA rule.
#pragma unroll
    for (int w = 0; w < NW; w++) {
        uint32_t hi = 0, lo = 0, valid = 0;
        int base = w * 32;
        if (base < m) {
            int cnt = min(32, m - base);
            valid = cnt >= 32 ? 0xffffffffu : ((1u << cnt) - 1u);
            uint32_t nmask = 0;
#pragma unroll
            for (int half = 0; half < 2; half++) {
                int b16 = base + 16 * half;
                if (b16 >= m) break;
                uint32_t cw = load16(job.arena, P.read_pos + (uint64_t)b16);
                // code k at bits (31-2k, 30-2k): reverse so code k sits at
                // bits (2k = high, 2k+1 = low), then unshuffle even/odd bits
                uint32_t x = __brev(cw);
                uint32_t e = x & 0x55555555u, o = (x >> 1) & 0x55555555u;
                e = (e | (e >> 1)) & 0x33333333u;
                e = (e | (e >> 2)) & 0x0f0f0f0fu;
                e = (e | (e >> 4)) & 0x00ff00ffu;
                e = (e | (e >> 8)) & 0x0000ffffu;
                o = (o | (o >> 1)) & 0x33333333u;
                o = (o | (o >> 2)) & 0x0f0f0f0fu;
                o = (o | (o >> 4)) & 0x00ff00ffu;
                o = (o | (o >> 8)) & 0x0000ffffu;
                hi |= e << (16 * half);
                lo |= o << (16 * half);
                if (P.n_read) nmask |= __brev(nmask16(iv, P.n_read, b16)) << (16 * half);
            }
            valid &= ~nmask;  // read N matches nothing
        }
        uint32_t a = ~hi & ~lo & valid, c = ~hi & lo & valid, g = hi & ~lo & valid,
                 tt = hi & lo & valid;
        uint32_t rows[4] = {a | g, c, g, tt | c};  // text A, C, G, T
        if (!rev) {
#pragma unroll
            for (int q = 0; q < 4; q++) peq[(q * NW + w) * bs + t] = rows[q];
            peq[(4 * NW + w) * bs + t] = 0u;
        } else {
            // reversed read: position i -> bit m-1-i; stored after all limbs
#pragma unroll
            for (int q = 0; q < 4; q++) peq[(q * NW + w) * bs + t] = rows[q];
        }
    }
    if (rev) {
        // Reverse each row as one m-bit vector (position i -> bit m-1-i):
        // bit-reverse over this pair's own nwp limbs (nwp*32 - m < 32 padding
        // bits), then shift the padding out.  Sources are re-read from shared
        // memory, where a runtime limb index costs nothing.
        const int nwp = (m + 31) >> 5;
        const int pad = nwp * 32 - m;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            uint32_t dst[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                uint32_t r0 = 0, r1 = 0;
                if (w < nwp) {
                    r0 = __brev(peq[(q * NW + (nwp - 1 - w)) * bs + t]);
                    if (w + 1 < nwp) r1 = __brev(peq[(q * NW + (nwp - 2 - w)) * bs + t]);
                }
                dst[w] = pad ? __funnelshift_r(r0, r1, pad) : r0;
            }
#pragma unroll
            for (int w = 0; w < NW; w++) peq[(q * NW + w) * bs + t] = dst[w];
        }
#pragma unroll
        for (int w = 0; w < NW; w++) peq[(4 * NW + w) * bs + t] = 0u;
    }
    uint32_t pv[NW], mv[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) {
        int lo = w * 32;
        pv[w] = m >= lo + 32 ? 0xffffffffu : (m > lo ? ((1u << (m - lo)) - 1u) : 0u);
        mv[w] = 0u;
    }
    const int topw = (m - 1) >> 5;
    const uint32_t topb = 1u << ((m - 1) & 31);
    int score = m, best = m;
    int64_t best_at = 0;
    const uint32_t hin = glob ? 1u : 0u;
    const esp_n_interval *tiv = iv + P.n_read;
    for (int64_t base = 0; base < n; base += 16) {
        int cnt = (int)min((int64_t)16, n - base);
        // text position of column index x: forward x, reversed n-1-x
        int64_t q0 = rev ? (n - base - 16) : base;  // first position of the 16-base window
        uint32_t cw, nm;
        if (rev && q0 < 0) {
            // short leading window of a reversed scan: fetch [0, 16) and shift
            cw = load16(job.arena, P.text_pos);
            nm = P.n_text ? nmask16(tiv, P.n_text, 0) : 0u;
            int sh = (int)(-q0);
            cw >>= 2 * sh;
            nm >>= sh;
            q0 = 0;
        } else {
            cw = load16(job.arena, P.text_pos + (uint64_t)q0);
            nm = P.n_text ? nmask16(tiv, P.n_text, q0) : 0u;
        }
#pragma unroll 4
        for (int x = 0; x < cnt; x++) {
            // forward: position base+x is slot x of the window; reversed:
            // position n-1-(base+x) is slot 15-x of the (right-aligned) window
            int slot = rev ? (15 - x) : x;
            uint32_t c = (cw >> (30 - 2 * slot)) & 3u;
            if ((nm >> (31 - slot)) & 1u) c = 4u;
            uint32_t eq[NW], xv[NW], s[NW], ph[NW], mh[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                eq[w] = peq[(c * NW + w) * bs + t];
                xv[w] = eq[w] | mv[w];
                s[w] = eq[w] & pv[w];
            }
            add_chain<NW>(s, s, pv);
            uint32_t hp = 0, hm = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                uint32_t xh = (s[w] ^ pv[w]) | xv[w];
                ph[w] = mv[w] | ~(xh | pv[w]);
                mh[w] = pv[w] & xh;
                if (w == topw) {
                    hp = ph[w] & topb;
                    hm = mh[w] & topb;
                }
            }
#pragma unroll
            for (int w = NW - 1; w >= 0; w--) {
                uint32_t phs = w ? __funnelshift_l(ph[w - 1], ph[w], 1) : ((ph[0] << 1) | hin);
                uint32_t mhs = w ? __funnelshift_l(mh[w - 1], mh[w], 1) : (mh[0] << 1);
                pv[w] = mhs | ~(xv[w] | phs);
                mv[w] = phs & xv[w];
            }
            score += (hp ? 1 : 0) - (hm ? 1 : 0);
            if (!glob && score < best) {
                best = score;
                best_at = base + x + 1;
            }
        }
    }
    if (glob) {
        res.dist = score > 0 ? score : 0;
        res.pos = 0;
    } else {
        res.dist = best;
        res.pos = rev ? (uint64_t)(n - best_at) : (uint64_t)best_at;
    }
    job.out[k] = res;
}

template <int NW>
__global__ void __launch_bounds__(MY_BLOCK) myers_kernel(MyersJob job) {
    extern __shared__ uint32_t smem[];
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < job.n_pairs;
         k += (uint64_t)gridDim.x * blockDim.x)
        myers_pair<NW>(job, (uint32_t)k, smem);
}

cudaError_t launch_myers(const MyersJob &job, int nw, int num_sms, cudaStream_t st) {
    if (job.n_pairs == 0) return cudaSuccess;
    size_t smem = (size_t)5 * nw * MY_BLOCK * sizeof(uint32_t);
    uint64_t need = (job.n_pairs + MY_BLOCK - 1) / MY_BLOCK;
    uint64_t cap = (uint64_t)num_sms * 16;
    int grid = (int)(need < cap ? need : cap);
    switch (nw) {
#define ESP_MY_CASE(W) \
    case W: myers_kernel<W><<<grid, MY_BLOCK, smem, st>>>(job); break;
        ESP_MY_CASE(1) ESP_MY_CASE(2) ESP_MY_CASE(3) ESP_MY_CASE(4)
        ESP_MY_CASE(5) ESP_MY_CASE(6) ESP_MY_CASE(7) ESP_MY_CASE(8)
#undef ESP_MY_CASE
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace esp
