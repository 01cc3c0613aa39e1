// bins.cu -- length-binned work list for the persistent DP kernels.
//
// Pairs are counting-sorted on the device by a 16-bit geometry key (band
// width bucket, read length bucket) in DESCENDING cost order, so that (a)
// the 32 pairs a warp takes from the queue share their loop trip counts and
// (b) the most expensive pairs start first (the tail of the launch is made
// of cheap pairs).  Three small kernels: histogram, scan, scatter; warp-
// aggregated atomics keep a single hot bin (uniform batches) cheap.
#include <cuda_runtime.h>

#include <cstdint>

#include "esp_internal.h"

namespace esp {

static constexpr int NBINS = 1 << 16;

// Key: larger = more expensive.  w = columns per row (band width or window),
// m = rows.  Both bucketed to 8 bits.
__device__ __forceinline__ uint32_t geometry_key(const esp_pair &P, int mode) {
    uint32_t m = P.read_len, n = P.win_len;
    uint32_t w;
    bool full = (mode == 0) ? (P.band_half < 0) : (n <= 30);
    if (full) {
        w = n;
    } else {
        uint32_t h = mode == 0 ? (uint32_t)P.band_half : 30u;
        uint64_t bw = 2ull * h + 1;
        w = (uint32_t)(bw < n ? bw : n);
    }
    uint32_t wb = w >= 1020 ? 255 : (w >> 2);
    uint32_t mb = m >= 2040 ? 255 : (m >> 3);
    return (wb << 8) | mb;
}

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

__global__ void bin_hist(const esp_pair *__restrict__ pairs, uint64_t n, int mode,
                         uint32_t *__restrict__ hist) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t key = geometry_key(pairs[i], mode);
        agg_add(hist, NBINS - 1 - key, nullptr);  // descending cost order
    }
}

// Exclusive scan of NBINS counters by one block of 1024 threads.
__global__ void __launch_bounds__(1024) bin_scan(uint32_t *__restrict__ hist) {
    __shared__ uint32_t part[1024];
    const int per = NBINS / 1024;
    uint32_t *h = hist + threadIdx.x * per;
    uint32_t s = 0;
#pragma unroll 1
    for (int k = 0; k < per; k++) s += h[k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
#pragma unroll 1
    for (int k = 0; k < per; k++) {
        uint32_t c = h[k];
        h[k] = run;
        run += c;
    }
}

__global__ void bin_scatter(const esp_pair *__restrict__ pairs, uint64_t n, int mode,
                            uint32_t *__restrict__ cursor, uint32_t *__restrict__ order) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t key = geometry_key(pairs[i], mode);
        uint32_t slot;
        agg_add(cursor, NBINS - 1 - key, &slot);
        order[slot] = (uint32_t)i;
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

size_t bin_scratch_bytes() { return (size_t)NBINS * sizeof(uint32_t); }

// Length classes of the binned list (descending cost): band/window width
// w >= 196, [100, 196), [52, 100), < 52 columns.  bounds[s], bounds[s+1] is
// class s; read from the scanned histogram before the scatter moves it.
__global__ void class_bounds(const uint32_t *__restrict__ hist, uint64_t n,
                             uint32_t *__restrict__ bounds) {
    if (threadIdx.x == 0) {
        const uint32_t first_key[3] = {(48u << 8) | 255u, (24u << 8) | 255u, (12u << 8) | 255u};
        bounds[0] = 0;
        for (int s = 0; s < 3; s++) bounds[s + 1] = hist[NBINS - 1 - first_key[s]];
        bounds[4] = (uint32_t)n;
    }
}

cudaError_t launch_binning(const esp_pair *pairs, uint64_t n, int mode, uint32_t *hist,
                           uint32_t *order, int num_sms, cudaStream_t st, uint32_t *bounds) {
    cudaError_t e = cudaMemsetAsync(hist, 0, bin_scratch_bytes(), st);
    if (e != cudaSuccess) return e;
    int grid = num_sms * 4;
    uint64_t need = (n + 255) / 256;
    if ((uint64_t)grid > need) grid = (int)(need ? need : 1);
    bin_hist<<<grid, 256, 0, st>>>(pairs, n, mode, hist);
    bin_scan<<<1, 1024, 0, st>>>(hist);
    if (bounds) class_bounds<<<1, 32, 0, st>>>(hist, n, bounds);
    bin_scatter<<<grid, 256, 0, st>>>(pairs, n, mode, hist, order);
    return cudaGetLastError();
}

}  // namespace esp
