// bins.cu -- length-binned work list for the persistent DP kernels.
//
// Pairs are counting-sorted on the device by a 20-bit geometry key (columns
// per row, rows; both exact below 1023) in DESCENDING cost order, so that
// (a) the 32 pairs a warp takes from the queue share their loop trip counts,
// (b) the most expensive pairs start first (the tail of the launch is made
// of cheap pairs) and (c) neighbours in the list usually have identical band
// geometry, which the two-pairs-per-thread kernel needs.  Kernels:
// histogram, a three-phase scan, scatter; warp-aggregated atomics keep a
// single hot bin (uniform batches) cheap.
#include <cuda_runtime.h>

#include <cstdint>

#include "esp_internal.h"

namespace esp {

static constexpr int KEY_BITS = 10;
static constexpr int NBINS = 1 << (2 * KEY_BITS);
static constexpr int SCAN_TILE = 1024;  // counters per block of the scan
static constexpr int SCAN_BLOCKS = NBINS / SCAN_TILE;

// Key: larger = more expensive.  m = rows; w = columns per row (band
// width or window) in band mode and extend_hint's full-matrix attempt
// (mode 2); in its banded first attempt (mode 1) the window length instead:
// every first attempt has width 61 (or the window, up to 30), so the window
// length orders them as well and, with the rows, pins their geometry
// wherever the hint offset follows from the lengths (read + 2h windows at
// offset h, flank segments at offset 0, fixed-shape reads).
__device__ __forceinline__ uint32_t geometry_key(const esp_pair &P, int mode) {
    uint32_t m = P.read_len, n = P.win_len;
    uint32_t w;
    bool full = (mode == 0) ? (P.band_half < 0) : (mode == 2 || n <= 30);
    if (full || mode == 1) {
        w = n;
    } else {
        uint64_t bw = 2ull * (uint32_t)P.band_half + 1;
        w = (uint32_t)(bw < n ? bw : n);
    }
    const uint32_t top = (1u << KEY_BITS) - 1;
    return ((w < top ? w : top) << KEY_BITS) | (m < top ? m : top);
}

// Entry k of the pairs to bin: k itself, or list[k] over *count entries.
struct BinInput {
    const uint32_t *list;   // null: pairs 0 .. n-1
    const uint32_t *count;  // device count of list entries (list only)
    __device__ __forceinline__ uint64_t size(uint64_t n) const { return list ? *count : n; }
    __device__ __forceinline__ uint32_t at(uint64_t k) const { return list ? list[k] : (uint32_t)k; }
};

__device__ __forceinline__ void agg_add(uint32_t *ctr, uint32_t key, uint32_t *slot) {
    // warp-aggregated atomicAdd on ctr[key]; returns each lane's slot
    uint32_t active = __activemask();
    uint32_t peers = __match_any_sync(active, key);
    int leader = __ffs(peers) - 1;
    int lane = threadIdx.x & 31;
    uint32_t rank = __popc(peers & ((1u << lane) - 1));
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (slot) *slot = base + rank;
}

__global__ void bin_hist(const esp_pair *__restrict__ pairs, uint64_t n, BinInput in, int mode,
                         uint32_t *__restrict__ hist) {
    const uint64_t cnt = in.size(n);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t pi = in.at(i);
        if (pi >= n) continue;  // never index past the batch
        uint32_t key = geometry_key(pairs[pi], mode);
        agg_add(hist, NBINS - 1 - key, nullptr);  // descending cost order
    }
}

// Exclusive scan of the NBINS counters in three phases: tile sums, a scan of
// the tile sums (one block), tile scans offset by their prefix.  part[] holds
// SCAN_BLOCKS words after the counters.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t *s_warp,
                                                       uint32_t &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    uint32_t wpre = 0;
    total = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t w = s_warp[k];
        if (k < wid) wpre += w;
        total += w;
    }
    return wpre + x - v;
}

// PAD: every bin's slot count rounded up to even, so that list positions
// 2k, 2k + 1 never straddle two bins; the spare slot of an odd bin holds
// NO_PAIR (the list is pre-filled with it).
__device__ __forceinline__ uint4 bin_counts(uint4 q, bool pad) {
    if (pad) {
        q.x += q.x & 1u;
        q.y += q.y & 1u;
        q.z += q.z & 1u;
        q.w += q.w & 1u;
    }
    return q;
}

template <bool PAD>
__global__ void __launch_bounds__(256) bin_scan_up(const uint32_t *__restrict__ hist,
                                                   uint32_t *__restrict__ part) {
    __shared__ uint32_t s_warp[8];
    uint4 q = bin_counts(
        reinterpret_cast<const uint4 *>(hist + (size_t)blockIdx.x * SCAN_TILE)[threadIdx.x], PAD);
    uint32_t total;
    block_excl_scan256(q.x + q.y + q.z + q.w, s_warp, total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// Also writes the list length (the sum of all slots) to *total.
__global__ void __launch_bounds__(1024) bin_scan_top(uint32_t *__restrict__ part,
                                                     uint32_t *__restrict__ total) {
    __shared__ uint32_t s[1024];
    uint32_t v = threadIdx.x < SCAN_BLOCKS ? part[threadIdx.x] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t y = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += y;
        __syncthreads();
    }
    if (threadIdx.x < SCAN_BLOCKS) part[threadIdx.x] = s[threadIdx.x] - v;
    if (threadIdx.x == 1023) *total = s[1023];
}

template <bool PAD>
__global__ void __launch_bounds__(256) bin_scan_down(uint32_t *__restrict__ hist,
                                                     const uint32_t *__restrict__ part) {
    __shared__ uint32_t s_warp[8];
    uint4 *tile = reinterpret_cast<uint4 *>(hist + (size_t)blockIdx.x * SCAN_TILE);
    uint4 q = bin_counts(tile[threadIdx.x], PAD);
    uint32_t total;
    uint32_t run = part[blockIdx.x] + block_excl_scan256(q.x + q.y + q.z + q.w, s_warp, total);
    uint4 r;
    r.x = run;
    r.y = r.x + q.x;
    r.z = r.y + q.y;
    r.w = r.z + q.z;
    tile[threadIdx.x] = r;
}

__global__ void bin_scatter(const esp_pair *__restrict__ pairs, uint64_t n, BinInput in, int mode,
                            uint32_t *__restrict__ cursor, uint32_t *__restrict__ order) {
    const uint64_t cnt = in.size(n);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t pi = in.at(i);
        if (pi >= n) continue;
        uint32_t key = geometry_key(pairs[pi], mode);
        uint32_t slot;
        agg_add(cursor, NBINS - 1 - key, &slot);
        order[slot] = pi;
    }
}

// Window width summed over rows 1..m (extend.rs:653-696).
__device__ uint64_t band_cells(uint32_t m, uint32_t n, int64_t off, int64_t half) {
    uint64_t cells = 0;
    for (uint32_t i = 1; i <= m; i++) {
        int64_t c = off + i;
        c = c < 1 ? 1 : (c > n ? n : c);
        int64_t lo = c - half > 1 ? c - half : 1;
        int64_t hi = c + half < (int64_t)n ? c + half : (int64_t)n;
        if (hi >= lo) cells += (uint64_t)(hi - lo + 1);
    }
    return cells;
}

__global__ void count_cells(const esp_pair *__restrict__ pairs,
                            const esp_extension *__restrict__ out, uint64_t n, int mode,
                            unsigned long long *cells) {
    uint64_t acc = 0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const esp_pair P = pairs[k];
        uint32_t m = P.read_len, w = P.win_len;
        if (m == 0 || w == 0) continue;
        if (mode == 0) {
            acc += P.band_half < 0 ? (uint64_t)m * w : band_cells(m, w, P.band_offset, P.band_half);
        } else if (w <= 30) {
            acc += (uint64_t)m * w;
        } else {
            acc += band_cells(m, w, P.band_offset, 30);
            if (out[k].escalated) acc += (uint64_t)m * w;
        }
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(cells, (unsigned long long)acc);
}

cudaError_t launch_count_cells(const esp_pair *pairs, const esp_extension *out, uint64_t n,
                               int mode, unsigned long long *cells, int num_sms,
                               cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    uint64_t need = (n + 255) / 256;
    int grid = (int)(need < (uint64_t)num_sms * 8 ? need : (uint64_t)num_sms * 8);
    count_cells<<<grid, 256, 0, st>>>(pairs, out, n, mode, cells);
    return cudaGetLastError();
}

size_t bin_scratch_bytes() { return (size_t)(NBINS + SCAN_BLOCKS) * sizeof(uint32_t); }

uint64_t bin_pad_slots(uint64_t n) { return n < (uint64_t)NBINS ? n : (uint64_t)NBINS; }

// Length classes of the binned list (descending cost): band/window width
// w >= 196, [100, 196), [52, 100), < 52 columns.  bounds[s], bounds[s+1] is
// class s; read from the scanned histogram before the scatter moves it.
__global__ void class_bounds(const uint32_t *__restrict__ hist, const uint32_t *__restrict__ total,
                             uint32_t *__restrict__ bounds) {
    if (threadIdx.x == 0) {
        const uint32_t top = (1u << KEY_BITS) - 1;
        const uint32_t first_w[3] = {195u, 99u, 51u};  // widest width of classes 1..3
        bounds[0] = 0;
        for (int s = 0; s < 3; s++)
            bounds[s + 1] = hist[NBINS - 1 - ((first_w[s] << KEY_BITS) | top)];
        bounds[4] = *total;
    }
}

cudaError_t launch_binning(const esp_pair *pairs, uint64_t n, int mode, uint32_t *hist,
                           uint32_t *order, int num_sms, cudaStream_t st, uint32_t *total,
                           uint32_t *bounds, bool pad, const uint32_t *list,
                           const uint32_t *list_count) {
    const BinInput in{list, list_count};
    cudaError_t e = cudaMemsetAsync(hist, 0, bin_scratch_bytes(), st);
    if (e == cudaSuccess && pad)
        e = cudaMemsetAsync(order, 0xff, (n + bin_pad_slots(n)) * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    int grid = num_sms * 4;
    uint64_t need = (n + 255) / 256;
    if ((uint64_t)grid > need) grid = (int)(need ? need : 1);
    bin_hist<<<grid, 256, 0, st>>>(pairs, n, in, mode, hist);
    if (pad) bin_scan_up<true><<<SCAN_BLOCKS, 256, 0, st>>>(hist, hist + NBINS);
    else bin_scan_up<false><<<SCAN_BLOCKS, 256, 0, st>>>(hist, hist + NBINS);
    bin_scan_top<<<1, 1024, 0, st>>>(hist + NBINS, total);
    if (pad) bin_scan_down<true><<<SCAN_BLOCKS, 256, 0, st>>>(hist, hist + NBINS);
    else bin_scan_down<false><<<SCAN_BLOCKS, 256, 0, st>>>(hist, hist + NBINS);
    if (bounds) class_bounds<<<1, 32, 0, st>>>(hist, total, bounds);
    bin_scatter<<<grid, 256, 0, st>>>(pairs, n, in, mode, hist, order);
    return cudaGetLastError();
}

}  // namespace esp
