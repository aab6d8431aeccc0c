// Batch preparation: per-read k-mer counts and their exclusive prefix (kofs),
// the map-tile -> read index, and the storage-independent hash kernel.
//
// A read of length L contributes max(0, L-K+1) k-mers; reads shorter than K
// contribute none, the way InserterProcessor skips them
// (processors.hh:304-331) after KmerIterator throws (kmeriterator.hh:72-74).
#include "gdbg_kernels.cuh"
#include "gdbg_launch.h"

namespace gdbg {

constexpr int SCAN_BLOCK = 1024;

// err == nullptr: check without reporting (the partials pass reports).
__device__ __forceinline__ uint64_t read_kmers(const uint64_t* __restrict__ off, uint64_t r,
                                               uint32_t K, uint64_t max_bases, uint32_t* err) {
    uint64_t a = __ldg(off + r), b = __ldg(off + r + 1);
    if (b < a || b > max_bases) {
        if (err) atomicOr(err, GDBG_ERR_BAD_OFFSETS);
        return 0;
    }
    uint64_t L = b - a;
    return L >= K ? L - K + 1 : 0;
}

// Inclusive block scan of one value per thread (SCAN_BLOCK threads).
__device__ __forceinline__ uint64_t block_inclusive_scan(uint64_t v, uint64_t* warp_sums) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
        uint64_t s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t t = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    if (wid > 0) v += warp_sums[wid - 1];
    return v;
}

// Per read: v.x = k-mers, v.y = warp tasks (ceil(k-mers / 32)).
__device__ __forceinline__ ulonglong2 read_counts(const uint64_t* __restrict__ off, uint64_t r,
                                                 uint32_t K, uint64_t max_bases, uint32_t* err) {
    uint64_t nk = read_kmers(off, r, K, max_bases, err);
    return make_ulonglong2(nk, (nk + TASK_KMERS - 1) / TASK_KMERS);
}

__global__ void __launch_bounds__(SCAN_BLOCK)
k_prefix_partials(const uint64_t* __restrict__ off, uint64_t n, uint32_t K, uint64_t max_bases,
                  uint64_t* __restrict__ partials, uint32_t* err) {
    __shared__ uint64_t ws[32], wt[32];
    uint64_t r = (uint64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    ulonglong2 v = r < n ? read_counts(off, r, K, max_bases, err) : make_ulonglong2(0, 0);
    uint64_t s = block_inclusive_scan(v.x, ws);
    uint64_t t = block_inclusive_scan(v.y, wt);
    if (threadIdx.x == SCAN_BLOCK - 1) {
        partials[2 * blockIdx.x] = s;
        partials[2 * blockIdx.x + 1] = t;
    }
}

// Each block first sums the (k-mer, task) totals of the blocks before it,
// so no separate pass scans the partials.
__global__ void __launch_bounds__(SCAN_BLOCK)
k_prefix_final(const uint64_t* __restrict__ off, uint64_t n, uint32_t K, uint64_t max_bases,
               const uint64_t* __restrict__ partials, uint64_t* __restrict__ kofs,
               uint64_t* __restrict__ tofs) {
    __shared__ uint64_t ws[32], wt[32];
    __shared__ uint64_t before_s[2];
    uint64_t pk = 0, pt = 0;
    for (uint32_t i = threadIdx.x; i < blockIdx.x; i += SCAN_BLOCK) {
        pk += partials[2 * i];
        pt += partials[2 * i + 1];
    }
    pk = block_inclusive_scan(pk, ws);
    pt = block_inclusive_scan(pt, wt);
    if (threadIdx.x == SCAN_BLOCK - 1) {
        before_s[0] = pk;
        before_s[1] = pt;
    }
    __syncthreads();
    uint64_t r = (uint64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    ulonglong2 v = r < n ? read_counts(off, r, K, max_bases, nullptr) : make_ulonglong2(0, 0);
    uint64_t s = block_inclusive_scan(v.x, ws) + before_s[0];
    uint64_t t = block_inclusive_scan(v.y, wt) + before_s[1];
    if (r < n) {
        kofs[r] = s - v.x;
        tofs[r] = t - v.y;
        if (r == n - 1) {
            kofs[n] = s;
            tofs[n] = t;
        }
    }
}

// One block does the whole prefix when the batch has at most SCAN_BLOCK reads.
__global__ void __launch_bounds__(SCAN_BLOCK)
k_prefix_small(const uint64_t* __restrict__ off, uint64_t n, uint32_t K, uint64_t max_bases,
               uint64_t* __restrict__ kofs, uint64_t* __restrict__ tofs, uint32_t* err) {
    __shared__ uint64_t ws[32], wt[32];
    const uint64_t r = threadIdx.x;
    ulonglong2 v = r < n ? read_counts(off, r, K, max_bases, err) : make_ulonglong2(0, 0);
    const uint64_t s = block_inclusive_scan(v.x, ws);
    const uint64_t t = block_inclusive_scan(v.y, wt);
    if (r < n) {
        kofs[r] = s - v.x;
        tofs[r] = t - v.y;
        if (r == n - 1) {
            kofs[n] = s;
            tofs[n] = t;
        }
    }
}

cudaError_t launch_kmer_prefix(const uint64_t* offsets, uint64_t n_reads, uint32_t K,
                               uint64_t max_bases, uint64_t* partials, uint64_t* kofs,
                               uint64_t* tofs, uint32_t* err, cudaStream_t st, int* launches) {
    if (n_reads == 0) {
        *launches = 0;
        cudaMemsetAsync(tofs, 0, sizeof(uint64_t), st);
        return cudaMemsetAsync(kofs, 0, sizeof(uint64_t), st);
    }
    if (n_reads <= SCAN_BLOCK) {
        k_prefix_small<<<1, SCAN_BLOCK, 0, st>>>(offsets, n_reads, K, max_bases, kofs, tofs, err);
        *launches = 1;
        return cudaGetLastError();
    }
    uint64_t nb = (n_reads + SCAN_BLOCK - 1) / SCAN_BLOCK;
    k_prefix_partials<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(offsets, n_reads, K, max_bases,
                                                           partials, err);
    k_prefix_final<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(offsets, n_reads, K, max_bases, partials,
                                                        kofs, tofs);
    *launches = 2;
    return cudaGetLastError();
}

// task_read[t] = read of warp task t, for t < n_tasks_cap.
__global__ void k_task_map(const uint64_t* __restrict__ tofs, uint64_t n, uint64_t cap,
                           uint32_t* __restrict__ task_read) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (uint64_t t = tofs[r], e = tofs[r + 1]; t < e && t < cap; ++t) task_read[t] = (uint32_t)r;
}

cudaError_t launch_task_map(const uint64_t* tofs, uint64_t n_reads, uint64_t cap,
                            uint32_t* task_read, cudaStream_t st) {
    if (n_reads == 0) return cudaSuccess;
    k_task_map<<<(unsigned)((n_reads + 255) / 256), 256, 0, st>>>(tofs, n_reads, cap, task_read);
    return cudaGetLastError();
}

// tile_read[t] = the read holding flattened k-mer t*MAP_TILE.
// Entries past n_tiles (the host's tile count) are not written.
__global__ void k_tile_map(const uint64_t* __restrict__ kofs, uint64_t n, uint64_t n_tiles,
                           uint32_t* __restrict__ tile_read) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    uint64_t a = kofs[r], b = kofs[r + 1];
    for (uint64_t t = (a + MAP_TILE - 1) / MAP_TILE; t * MAP_TILE < b && t < n_tiles; ++t)
        tile_read[t] = (uint32_t)r;
}

cudaError_t launch_tile_map(const uint64_t* kofs, uint64_t n_reads, uint64_t n_tiles,
                            uint32_t* tile_read, cudaStream_t st) {
    if (n_reads == 0) return cudaSuccess;
    k_tile_map<<<(unsigned)((n_reads + 255) / 256), 256, 0, st>>>(kofs, n_reads, n_tiles, tile_read);
    return cudaGetLastError();
}

cudaError_t launch_hashes(bool canonical, cudaStream_t st, const BatchView& b,
                          const HashParams& hp, uint64_t* values, uint64_t* fw, uint64_t* rc) {
    constexpr int H = 4;
    uint64_t n_threads = (b.n_kmers + H - 1) / H;
    if (n_threads == 0) return cudaSuccess;
    unsigned grid = (unsigned)((n_threads + BLOCK - 1) / BLOCK);
    if (canonical) k_hashes<true, H><<<grid, BLOCK, 0, st>>>(b, hp, values, fw, rc);
    else k_hashes<false, H><<<grid, BLOCK, 0, st>>>(b, hp, values, fw, rc);
    return cudaGetLastError();
}

}  // namespace gdbg
