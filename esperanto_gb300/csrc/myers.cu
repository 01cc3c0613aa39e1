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

// 16 text codes of one window in processing order: the code of the first
// column in bits 31:30, its N flag in bit 31 of `n`.
struct CodeWin {
    uint32_t c, n;
};

// Split 16 packed 2-bit codes (code k at bits 31-2k, 30-2k) into a high-bit
// and a low-bit mask with position k at bit k.
__device__ __forceinline__ void unshuffle16(uint32_t cw, uint32_t &hi, uint32_t &lo) {
    uint32_t x = __brev(cw);  // code k -> bits 2k (high), 2k+1 (low)
    uint32_t e = x & 0x55555555u, o = (x >> 1) & 0x55555555u;
    e = (e | (e >> 1)) & 0x33333333u;
    e = (e | (e >> 2)) & 0x0f0f0f0fu;
    e = (e | (e >> 4)) & 0x00ff00ffu;
    e = (e | (e >> 8)) & 0x0000ffffu;
    o = (o | (o >> 1)) & 0x33333333u;
    o = (o | (o >> 2)) & 0x0f0f0f0fu;
    o = (o | (o >> 4)) & 0x00ff00ffu;
    o = (o | (o >> 8)) & 0x0000ffffu;
    hi = e;
    lo = o;
}

// Pattern rows of 32 read positions starting at position `b` (may be
// negative: positions < 0 are absent): high/low code bits and the mask of
// real ACGT positions (bit k <-> position b + k).
__device__ __forceinline__ void read_limb(const MyersJob &job, const esp_myers_pair &P,
                                          const esp_n_interval *iv, int m, int b, uint32_t &hi,
                                          uint32_t &lo, uint32_t &real) {
    hi = lo = real = 0;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        int s = b + 16 * half;  // first position of this 16-position half
        if (s + 16 <= 0 || s >= m) continue;
        int start = s < 0 ? 0 : s;
        int skip = start - s;  // leading absent positions (s < 0)
        uint32_t cw = load16(job.arena, P.read_pos + (uint64_t)start);
        uint32_t nm = P.n_read ? nmask16(iv, P.n_read, start) : 0u;
        uint32_t h, l;
        unshuffle16(cw, h, l);
        uint32_t nb = __brev(nm) & 0xffffu;  // position start + k -> bit k
        int cnt = min(16 - skip, m - start);
        uint32_t v = (cnt >= 16 ? 0xffffu : ((1u << cnt) - 1u)) & ~nb;  // read N matches nothing
        int sh = 16 * half + skip;
        hi |= h << sh;
        lo |= l << sh;
        real |= v << sh;
    }
}

// EA Peq rows for text A, C, G, T from one limb's code bits.
__device__ __forceinline__ void ea_rows(uint32_t hi, uint32_t lo, uint32_t real,
                                        uint32_t (&rows)[4]) {
    uint32_t a = ~hi & ~lo & real, c = ~hi & lo & real, g = hi & ~lo & real,
             tt = hi & lo & real;
    rows[0] = a | g;   // text A: read A or G
    rows[1] = c;       // text C: read C
    rows[2] = g;       // text G: read G
    rows[3] = tt | c;  // text T: read T or C
}

// One pair.  flags: MYF_REVERSE (best start: read and text both reversed,
// myers_ea.rs:158-185), MYF_GLOBAL (engine global: leading column +1 per text
// base, engine/src/myers.rs:151-169).
//
// TOP (every non-global search): the m pattern rows occupy the TOP m bits of
// the NW*32-bit vector, so the last row is always bit 31 of limb NW-1 and the
// score update needs no runtime limb select.  The bits below are virtual
// rows that match every text base and start with vertical delta 0: they keep
// D = 0 in every column (their horizontal deltas are 0, they never carry into
// the real rows and they shift 0 into real row 0), which is the semi-global
// boundary the real rows had with hin = 0.  Global search (hin = +1) keeps
// the pattern in the low bits.
template <int NW, bool TOP>
__device__ void myers_pair(const MyersJob &job, uint32_t k, uint32_t *__restrict__ peq) {
    const esp_myers_pair P = job.pairs[k];
    const int m = (int)P.read_len;
    const int64_t n = P.text_len;
    const bool rev = job.flags & MYF_REVERSE;
    const bool glob = !TOP;
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
    const int off = TOP ? NW * 32 - m : 0;  // virtual rows below the pattern
    uint32_t pv[NW], mv[NW];
    // Peq rows: text code 0..3, row 4 (text N): virtual rows only.
    if (!rev) {
        // forward: limb w bit k <-> read position w*32 + k - off
#pragma unroll
        for (int w = 0; w < NW; w++) {
            uint32_t hi, lo, real;
            read_limb(job, P, iv, m, w * 32 - off, hi, lo, real);
            uint32_t rows[4];
            ea_rows(hi, lo, real, rows);
            const int vb = off - w * 32;  // virtual bits of this limb: [0, vb)
            const uint32_t virt = !TOP || vb <= 0 ? 0u : (vb >= 32 ? 0xffffffffu : (1u << vb) - 1u);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                peq[(q * NW + w) * bs + t] = rows[q] | virt;
                peq[((4 + q) * NW + w) * bs + t] = virt;  // text N: virtual rows only
            }
            // pattern rows start with vertical delta +1 (D[i][0] = i)
            if (TOP) {
                pv[w] = ~virt;
            } else {
                const int lim = m - w * 32;
                pv[w] = lim >= 32 ? 0xffffffffu : (lim > 0 ? (1u << lim) - 1u : 0u);
            }
            mv[w] = 0u;
        }
    } else {
        // reversed (TOP only): bottom-aligned forward limbs F (position p at
        // bit p) reversed as one NW*32-bit vector: position p -> bit
        // NW*32 - 1 - p, i.e. R[w] = brev(F[NW-1-w]); the padding above m
        // lands in the virtual bits [0, off).
        uint32_t F[4][NW];
#pragma unroll
        for (int w = 0; w < NW; w++) {
            uint32_t hi, lo, real;
            read_limb(job, P, iv, m, w * 32, hi, lo, real);
            uint32_t rows[4];
            ea_rows(hi, lo, real, rows);
#pragma unroll
            for (int q = 0; q < 4; q++) F[q][w] = rows[q];
        }
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const int vb = off - w * 32;
            const uint32_t virt = vb <= 0 ? 0u : (vb >= 32 ? 0xffffffffu : (1u << vb) - 1u);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                peq[(q * NW + w) * bs + t] = __brev(F[q][NW - 1 - w]) | virt;
                peq[((4 + q) * NW + w) * bs + t] = virt;
            }
            pv[w] = ~virt;
            mv[w] = 0u;
        }
    }
    const int topw = (m - 1) >> 5;  // global layout only
    const uint32_t topb = 1u << ((m - 1) & 31);
    int score = m, best = m;
    uint32_t best_at = 0, col = 0;
    const uint32_t hin = glob ? 1u : 0u;
    const esp_n_interval *tiv = iv + P.n_read;
    for (int64_t base = 0; base < n; base += 16) {
        int cnt = (int)min((int64_t)16, n - base);
        CodeWin win;
        if (!rev) {
            win.c = load16(job.arena, P.text_pos + (uint64_t)base);
            win.n = P.n_text ? nmask16(tiv, P.n_text, base) : 0u;
        } else {
            // right-aligned window [n-base-16, n-base): slot 15 first
            int64_t q0 = n - base - 16;
            uint32_t cw, nm;
            if (q0 < 0) {
                cw = load16(job.arena, P.text_pos);
                nm = P.n_text ? nmask16(tiv, P.n_text, 0) : 0u;
                int sh = (int)(-q0);
                cw >>= 2 * sh;
                nm >>= sh;
            } else {
                cw = load16(job.arena, P.text_pos + (uint64_t)q0);
                nm = P.n_text ? nmask16(tiv, P.n_text, q0) : 0u;
            }
            uint32_t x = __brev(cw);  // slot s -> bits 2s (high), 2s+1 (low)
            win.c = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
            win.n = __brev(nm) << 16;
        }
#pragma unroll 4
        for (int x = 0; x < cnt; x++) {
            uint32_t c = (win.c >> 30) | ((win.n >> 29) & 4u);  // text N: rows 4..7
            win.c <<= 2;
            win.n <<= 1;
            const uint32_t *pe = peq + (c * NW) * bs + t;
            uint32_t xv[NW], s[NW], ph[NW], mh[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                uint32_t eq = pe[w * bs];
                xv[w] = eq | mv[w];
                s[w] = eq & pv[w];
            }
            add_chain<NW>(s, s, pv);
#pragma unroll
            for (int w = 0; w < NW; w++) {
                uint32_t xh = (s[w] ^ pv[w]) | xv[w];
                ph[w] = mv[w] | ~(xh | pv[w]);
                mh[w] = pv[w] & xh;
            }
            int d;
            if (TOP) {
                d = (int)(ph[NW - 1] >> 31) - (int)(mh[NW - 1] >> 31);
            } else {
                uint32_t hp = 0, hm = 0;
#pragma unroll
                for (int w = 0; w < NW; w++) {
                    if (w == topw) {
                        hp = ph[w] & topb;
                        hm = mh[w] & topb;
                    }
                }
                d = (hp ? 1 : 0) - (hm ? 1 : 0);
            }
#pragma unroll
            for (int w = NW - 1; w >= 0; w--) {
                uint32_t phs = w ? __funnelshift_l(ph[w - 1], ph[w], 1) : ((ph[0] << 1) | hin);
                uint32_t mhs = w ? __funnelshift_l(mh[w - 1], mh[w], 1) : (mh[0] << 1);
                pv[w] = mhs | ~(xv[w] | phs);
                mv[w] = phs & xv[w];
            }
            score += d;
            col++;
            if (TOP && score < best) {
                best = score;
                best_at = col;
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

template <int NW, bool TOP>
__global__ void __launch_bounds__(MY_BLOCK) myers_kernel(MyersJob job) {
    extern __shared__ uint32_t smem[];
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < job.n_pairs;
         k += (uint64_t)gridDim.x * blockDim.x)
        myers_pair<NW, TOP>(job, (uint32_t)k, smem);
}

cudaError_t launch_myers(const MyersJob &job, int nw, int num_sms, cudaStream_t st) {
    if (job.n_pairs == 0) return cudaSuccess;
    size_t smem = (size_t)8 * nw * MY_BLOCK * sizeof(uint32_t);

    uint64_t need = (job.n_pairs + MY_BLOCK - 1) / MY_BLOCK;
    uint64_t cap = (uint64_t)num_sms * 16;
    int grid = (int)(need < cap ? need : cap);
    switch (nw) {
#define ESP_MY_CASE(W)                                                   \
    case W:                                                              \
        if (job.flags & MYF_GLOBAL)                                      \
            myers_kernel<W, false><<<grid, MY_BLOCK, smem, st>>>(job);   \
        else                                                             \
            myers_kernel<W, true><<<grid, MY_BLOCK, smem, st>>>(job);    \
        break;
        ESP_MY_CASE(1) ESP_MY_CASE(2) ESP_MY_CASE(3) ESP_MY_CASE(4)
        ESP_MY_CASE(5) ESP_MY_CASE(6) ESP_MY_CASE(7) ESP_MY_CASE(8)
#undef ESP_MY_CASE
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace esp
