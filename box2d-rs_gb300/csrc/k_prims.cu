/*
 * k_prims.cu — device-wide exclusive scan and stable LSD radix sort.
 *
 * Both take the element count from device memory (d_n), so a step can chain them
 * after kernels that produce a variable number of items without a host round trip;
 * grids are sized for the capacity and tiles past n do no work.
 *
 * Radix sort: 8-bit digits, tiles of 2048 items per 256-thread block. A pass is
 *   1. per-tile digit histograms, stored digit-major (hist[d * tiles + t]),
 *   2. an exclusive scan of that array, which yields each (digit, tile) output base,
 *   3. a stable scatter: the tile is walked in 8 rounds of 256 items; inside a warp
 *      __match_any_sync groups equal digits, and per-warp counts are prefixed across
 *      the 8 warps in shared memory, so every item's rank preserves input order.
 */
#include <algorithm>
#include <mutex>
#include <vector>

#include "b2g_internal.h"
#include "b2g_sync.cuh"

namespace b2g {

unsigned long long g_kernel_launches = 0;

int current_sm_count() {
    static std::mutex m;
    static std::vector<int> counts;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    std::lock_guard<std::mutex> lock(m);
    if ((int)counts.size() <= dev) counts.resize((size_t)dev + 1, 0);
    if (counts[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return 1;
        counts[dev] = n;
    }
    return counts[dev];
}

namespace {
constexpr int kScanBlock = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;
constexpr int kSortBlock = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortBlock * kSortItems;

__device__ __forceinline__ int load_n(const int* d_n, int max_n) {
    if (!d_n) return max_n;
    int n = *d_n;
    return n < max_n ? n : max_n;
}

/* block-wide exclusive scan of one value per thread; returns the block total in *total */
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < nwarps ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;  /* inclusive */
    }
    __syncthreads();
    uint32_t warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[nwarps - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, const int* d_n, int max_n,
                             uint32_t* __restrict__ tile_sums) {
    pdl_entry();
    const int n = load_n(d_n, max_n);
    const int base = blockIdx.x * kScanTile;
    if (base >= n) {
        if (threadIdx.x == 0) tile_sums[blockIdx.x] = 0;
        return;
    }
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        int idx = base + threadIdx.x * kScanItems + i;
        v[i] = idx < n ? in[idx] : 0u;
        sum += v[i];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(sum, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        int idx = base + threadIdx.x * kScanItems + i;
        if (idx < n) out[idx] = off;
        off += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

/* one block scans all tile sums (looping over chunks), writes the grand total */
__global__ void k_scan_sums(uint32_t* tile_sums, int tiles, int* d_total) {
    pdl_entry();
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < tiles; base += blockDim.x) {
        int i = base + threadIdx.x;
        uint32_t v = i < tiles ? tile_sums[i] : 0u;
        uint32_t total;
        uint32_t ex = block_exclusive_scan(v, &total);
        if (i < tiles) tile_sums[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && d_total) *d_total = (int)carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, const int* d_n, int max_n, const uint32_t* __restrict__ tile_sums) {
    pdl_entry();
    const int n = load_n(d_n, max_n);
    const int base = blockIdx.x * kScanTile;
    if (base >= n) return;
    const uint32_t add = tile_sums[blockIdx.x];
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        int idx = base + i;
        if (idx < n) out[idx] += add;
    }
}

__global__ void k_sort_hist(const unsigned long long* __restrict__ keys, const int* d_n, int max_n, int shift,
                            uint32_t* __restrict__ hist, int tiles) {
    __shared__ uint32_t h[256];
    const int n = load_n(d_n, max_n);
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortBlock) {
        int idx = base + i;
        if (idx < n) atomicAdd(&h[(unsigned)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_sort_scatter(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                               unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, const int* d_n,
                               int max_n, int shift, const uint32_t* __restrict__ offsets, int tiles) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_warp[8][256];
    const int n = load_n(d_n, max_n);
    const int tile_base = blockIdx.x * kSortTile;
    if (tile_base >= n) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s_base[threadIdx.x] = offsets[threadIdx.x * tiles + blockIdx.x];
    s_run[threadIdx.x] = 0;
    for (int w = 0; w < 8; ++w) s_warp[w][threadIdx.x] = 0;
    __syncthreads();
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = tile_base + r * kSortBlock + threadIdx.x;
        const bool valid = idx < n;
        unsigned long long k = 0;
        uint32_t v = 0;
        uint32_t d = 256u + (uint32_t)lane;  /* distinct dummy digits for invalid lanes */
        if (valid) {
            k = kin[idx];
            v = vin[idx];
            d = (uint32_t)(k >> shift) & 255u;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = (uint32_t)__popc(peers & lt_mask);
        const bool leader = (peers & lt_mask) == 0u;
        if (valid && leader) s_warp[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        {
            /* thread t owns digit t: prefix its count across the 8 warps */
            const int dd = threadIdx.x;
            uint32_t run = s_run[dd];
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                uint32_t c = s_warp[w][dd];
                s_warp[w][dd] = run;
                run += c;
            }
            s_run[dd] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = s_base[d] + s_warp[warp][d] + rank;
            if (dst < (uint32_t)n) {  /* always true for a correct scan; keeps writes in bounds */
                kout[dst] = k;
                vout[dst] = v;
            }
        }
        __syncthreads();
        for (int w = 0; w < 8; ++w) s_warp[w][threadIdx.x] = 0;
        __syncthreads();
    }
}

/* ---- single-launch cooperative radix sort ---- */

/* Stable scatter of one 2048-item tile given its per-digit output bases in s_base. */
__device__ void scatter_tile(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                             unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, int n, int shift,
                             int tile_base, const uint32_t* s_base, uint32_t* s_run, uint32_t (*s_warp)[256]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s_run[threadIdx.x] = 0;
    for (int w = 0; w < 8; ++w) s_warp[w][threadIdx.x] = 0;
    __syncthreads();
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = tile_base + r * kSortBlock + threadIdx.x;
        const bool valid = idx < n;
        unsigned long long k = 0;
        uint32_t v = 0;
        uint32_t d = 256u + (uint32_t)lane;
        if (valid) {
            k = kin[idx];
            v = vin[idx];
            d = (uint32_t)(k >> shift) & 255u;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = (uint32_t)__popc(peers & lt_mask);
        if (valid && (peers & lt_mask) == 0u) s_warp[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        {
            const int dd = threadIdx.x;
            uint32_t run = s_run[dd];
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                uint32_t c = s_warp[w][dd];
                s_warp[w][dd] = run;
                run += c;
            }
            s_run[dd] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = s_base[d] + s_warp[warp][d] + rank;
            if (dst < (uint32_t)n) {
                kout[dst] = k;
                vout[dst] = v;
            }
        }
        __syncthreads();
        for (int w = 0; w < 8; ++w) s_warp[w][threadIdx.x] = 0;
        __syncthreads();
    }
}

/* 256-bin histogram of one tile into s_cnt (block-wide) */
__device__ void tile_histogram(const unsigned long long* __restrict__ keys, int n, int shift, int tile_base, uint32_t* s_cnt) {
    s_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < kSortTile; i += kSortBlock) {
        const int idx = tile_base + i;
        if (idx < n) atomicAdd(&s_cnt[(unsigned)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
}

/* Between one tile and kRankSort pairs, the sort is a rank count instead of the multi-block radix
 * sort (whose two grid barriers per 8-bit pass dominate a few thousand keys): a block takes one
 * tile x of keys and a slice of the tiles y; each thread counts, for its key of tile x, the keys of
 * those tiles that precede it in (key, input position) order and adds the count to the key's rank
 * (one atomic per key and slice); the keys then go to their ranks. The order is the radix sort's
 * (stable: equal keys keep their input order). A fixed grid of kRankBlocks is mapped onto the
 * tiles and slices of the actual count. */
constexpr int kRankSort = 8192;  /* the count is quadratic: beyond this the radix sort is faster */
constexpr int kRankTile = 256;
constexpr int kRankBlocks = 1024;

__global__ void __launch_bounds__(kRankTile) k_rank_count(const unsigned long long* __restrict__ keys, const int* d_n,
                                                          int max_n, uint32_t* rank, int* cnt) {
    pdl_entry();
    if (world_aborted(cnt)) return;
    const int n = load_n(d_n, max_n);
    if (n <= kSortTile || n > kRankSort) return;
    __shared__ unsigned long long s_k[kRankTile];
    const int tiles = (n + kRankTile - 1) / kRankTile;
    const int slices = max(1, min(tiles, (int)gridDim.x / tiles));
    if ((int)blockIdx.x >= tiles * slices) return;
    const int tx = blockIdx.x % tiles, sl = blockIdx.x / tiles;
    const int per = (tiles + slices - 1) / slices;
    const int y0 = sl * per, y1 = min(tiles, y0 + per);
    const int j = tx * kRankTile + threadIdx.x;
    const unsigned long long kj = j < n ? keys[j] : 0ull;
    uint32_t r = 0;
    for (int ty = y0; ty < y1; ++ty) {
        const int i0 = ty * kRankTile;
        const int m = min(kRankTile, n - i0);
        __syncthreads();  /* the previous tile's keys are no longer read */
        if (threadIdx.x < m) s_k[threadIdx.x] = keys[i0 + threadIdx.x];
        __syncthreads();
        for (int i = 0; i < m; ++i) {
            const unsigned long long ki = s_k[i];
            r += (ki < kj || (ki == kj && i0 + i < j)) ? 1u : 0u;
        }
    }
    if (j < n && r) atomicAdd(&rank[j], r);
}

__global__ void k_rank_scatter(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                               unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, const int* d_n,
                               int max_n, const uint32_t* rank, int* cnt) {
    pdl_entry();
    if (world_aborted(cnt)) return;
    const int n = load_n(d_n, max_n);
    if (n <= kSortTile || n > kRankSort) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t r = rank[j];
        if (r < (uint32_t)n) {
            kout[r] = kin[j];
            vout[r] = vin[j];
        }
    }
}

__global__ void k_rank_copy(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                            unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, const int* d_n, int max_n,
                            int* cnt) {
    pdl_entry();
    if (world_aborted(cnt)) return;
    const int n = load_n(d_n, max_n);
    if (n <= kSortTile || n > kRankSort) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        kout[j] = kin[j];
        vout[j] = vin[j];
    }
}

__global__ void __launch_bounds__(kSortBlock) k_radix_coop(unsigned long long* ka, uint32_t* va, unsigned long long* kb,
                                                           uint32_t* vb, const int* d_n, int max_n, int bits,
                                                           uint32_t* hist, int* cnt) {
    if (world_aborted(cnt)) return;
    grid_barrier_start();
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_warp[8][256];
    __shared__ uint32_t s_cnt[256];
    const int n = load_n(d_n, max_n);
    const int passes = (bits + 7) / 8;
    if (n <= 0 || passes <= 0) return;
    if (n > kSortTile && n <= kRankSort && max_n > kSortTile) return;  /* the rank count sorted it */
    if (n <= kSortTile) {
        /* one tile: block 0 sorts alone, synchronising with __syncthreads only */
        if (blockIdx.x != 0) return;
        unsigned long long *kin = ka, *kout = kb;
        uint32_t *vin = va, *vout = vb;
        for (int p = 0; p < passes; ++p) {
            tile_histogram(kin, n, 8 * p, 0, s_cnt);
            uint32_t total;
            const uint32_t ex = block_exclusive_scan(s_cnt[threadIdx.x], &total);
            s_base[threadIdx.x] = ex;
            __syncthreads();
            scatter_tile(kin, vin, kout, vout, n, 8 * p, 0, s_base, s_run, s_warp);
            __syncthreads();
            unsigned long long* tk = kin; kin = kout; kout = tk;
            uint32_t* tv = vin; vin = vout; vout = tv;
        }
        if (kin != ka)
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                ka[i] = kin[i];
                va[i] = vin[i];
            }
        return;
    }
    const int tiles = (n + kSortTile - 1) / kSortTile;
    unsigned long long *kin = ka, *kout = kb;
    uint32_t *vin = va, *vout = vb;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        /* H: per-tile digit counts, tile-major */
        for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
            tile_histogram(kin, n, shift, t * kSortTile, s_cnt);
            hist[(size_t)t * 256 + threadIdx.x] = s_cnt[threadIdx.x];
            __syncthreads();
        }
        if (!grid_barrier(cnt)) return;
        /* X: a block with tiles derives its digit bases itself (thread d sums digit d over the
         * tiles: the digit's total and the counts of the tiles before each of its own), then
         * scatters its tiles stably; no separate scan phase and barrier */
        if ((int)blockIdx.x < tiles) {
            const int d = threadIdx.x;
            uint32_t tot = 0;
#pragma unroll 8
            for (int t = 0; t < tiles; ++t) tot += hist[(size_t)t * 256 + d];
            uint32_t total;
            const uint32_t digit_base = block_exclusive_scan(tot, &total);
            uint32_t before = 0;
            int next = 0;
            for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
                for (; next < t; ++next) before += hist[(size_t)next * 256 + d];
                s_base[d] = digit_base + before;
                __syncthreads();
                scatter_tile(kin, vin, kout, vout, n, shift, t * kSortTile, s_base, s_run, s_warp);
                __syncthreads();
            }
        }
        if (!grid_barrier(cnt)) return;
        unsigned long long* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
    }
    if (kin != ka) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            ka[i] = kin[i];
            va[i] = vin[i];
        }
    }
}

__global__ void k_copy_pairs(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                             unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, const int* d_n, int max_n) {
    const int n = load_n(d_n, max_n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kout[i] = kin[i];
        vout[i] = vin[i];
    }
}
}  // namespace

size_t scan_tmp_size(int max_n) { return (size_t)((max_n + kScanTile - 1) / kScanTile + 1); }

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, const int* d_n, int max_n, uint32_t* tmp, int* d_total,
                        cudaStream_t s) {
    const int tiles = (max_n + kScanTile - 1) / kScanTile;
    if (tiles == 0) return;
    launch_pdl(k_scan_tiles, tiles, kScanBlock, 0, s, in, out, d_n, max_n, tmp); B2G_LAUNCHED(1);
    launch_pdl(k_scan_sums, 1, 1024, 0, s, tmp, tiles, d_total); B2G_LAUNCHED(1);
    launch_pdl(k_scan_add, tiles, kScanBlock, 0, s, out, d_n, max_n, (const uint32_t*)tmp); B2G_LAUNCHED(1);
}

void radix_sort_pairs_coop(unsigned long long* key_a, uint32_t* val_a, unsigned long long* key_b, uint32_t* val_b,
                           const int* d_n, int max_n, int bits, uint32_t* hist, int* cnt, cudaStream_t s, int num_sms,
                           bool zero_or_max) {
    static int per_sm = 0;
    if (!per_sm) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_radix_coop, kSortBlock, 0);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 2) per_sm = 2;
    }
    /* one block per SM keeps the grid barrier short; per_sm only guards co-residency */
    const int blocks = num_sms;
    if (max_n > kSortTile && (!zero_or_max || max_n <= kRankSort)) {
        /* the rank count for inputs between one tile and kRankSort keys (each kernel checks n) */
        const int m = std::min(max_n, kRankSort);
        const int tiles = (m + kRankTile - 1) / kRankTile;
        cudaMemsetAsync(hist, 0, (size_t)m * sizeof(uint32_t), s);
        launch_pdl(k_rank_count, kRankBlocks, kRankTile, 0, s, (const unsigned long long*)key_a, d_n, max_n, hist, cnt);
        launch_pdl(k_rank_scatter, tiles, kRankTile, 0, s, (const unsigned long long*)key_a, (const uint32_t*)val_a,
                   key_b, val_b, d_n, max_n, (const uint32_t*)hist, cnt);
        launch_pdl(k_rank_copy, tiles, kRankTile, 0, s, (const unsigned long long*)key_b, (const uint32_t*)val_b, key_a,
                   val_a, d_n, max_n, cnt);
        B2G_LAUNCHED(3);
    }
    void* args[] = {&key_a, &val_a, &key_b, &val_b, (void*)&d_n, &max_n, &bits, &hist, &cnt};
    cudaMemsetAsync(cnt + CNT_BARRIER, 0, sizeof(int), s);
    cudaLaunchCooperativeKernel((const void*)k_radix_coop, dim3(blocks), dim3(kSortBlock), args, 0, s);
    B2G_LAUNCHED(1);
}

size_t radix_sort_hist_size(int max_n) {
    const int tiles = (max_n + kSortTile - 1) / kSortTile;
    /* the rank count uses the first kRankSort entries */
    return std::max((size_t)tiles * 256 * 2 + scan_tmp_size(tiles * 256) + 16, (size_t)kRankSort);
}

void radix_sort_pairs(unsigned long long* key_a, uint32_t* val_a, unsigned long long* key_b, uint32_t* val_b,
                      const int* d_n, int max_n, int bits, uint32_t* hist, cudaStream_t s) {
    const int tiles = (max_n + kSortTile - 1) / kSortTile;
    if (tiles == 0 || bits <= 0) return;
    uint32_t* h = hist;
    uint32_t* off = hist + (size_t)tiles * 256;
    uint32_t* tmp = off + (size_t)tiles * 256;
    int passes = (bits + 7) / 8;
    unsigned long long* kin = key_a;
    uint32_t* vin = val_a;
    unsigned long long* kout = key_b;
    uint32_t* vout = val_b;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_sort_hist<<<tiles, kSortBlock, 0, s>>>(kin, d_n, max_n, shift, h, tiles); B2G_LAUNCHED(1);
        scan_exclusive_u32(h, off, nullptr, tiles * 256, tmp, nullptr, s);
        k_sort_scatter<<<tiles, kSortBlock, 0, s>>>(kin, vin, kout, vout, d_n, max_n, shift, off, tiles); B2G_LAUNCHED(1);
        unsigned long long* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
    }
    if (kin != key_a) {
        k_copy_pairs<<<grid_for(max_n, 256, 4096), 256, 0, s>>>(kin, vin, key_a, val_a, d_n, max_n); B2G_LAUNCHED(1);
    }
}

}  // namespace b2g
