// Launchers for the bucketed insert path (kernels in gdbg_bucket.cuh).
#include <algorithm>

#include "gdbg_bucket.cuh"
#include "gdbg_launch.h"

namespace gdbg {

cudaError_t launch_bucket_emit(bool canonical, cudaStream_t st, const BatchView& b,
                               const HashParams& hp, const TableParams& tp, const BucketParams& bp) {
    const uint64_t warps = b.task_cap;
    uint64_t grid = (warps * 32 + BK_EMIT_BLOCK - 1) / BK_EMIT_BLOCK;
    if (grid > 152 * 64) grid = 152 * 64;
    if (grid == 0) return cudaSuccess;
    if (canonical) k_bkt_emit<true><<<(unsigned)grid, BK_EMIT_BLOCK, 0, st>>>(b, hp, tp, bp);
    else k_bkt_emit<false><<<(unsigned)grid, BK_EMIT_BLOCK, 0, st>>>(b, hp, tp, bp);
    return cudaGetLastError();
}

cudaError_t launch_bucket_hist(uint32_t n_tiles, cudaStream_t st, const BucketParams& bp) {
    if (n_tiles == 0) return cudaSuccess;
    k_bkt_hist<<<n_tiles, BK_TB, 0, st>>>(bp);
    return cudaGetLastError();
}

cudaError_t launch_bucket_scatter(bool last, uint32_t n_tiles, cudaStream_t st,
                                  const BucketParams& bp, uint32_t* start) {
    if (n_tiles == 0) return cudaSuccess;
    const size_t smem = bk_scatter_smem();
    cudaError_t e;
    if (last) {
        e = cudaFuncSetAttribute(k_bkt_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_bkt_scatter<true><<<n_tiles, BK_TB, smem, st>>>(bp, start);
    } else {
        e = cudaFuncSetAttribute(k_bkt_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_bkt_scatter<false><<<n_tiles, BK_TB, smem, st>>>(bp, start);
    }
    return cudaGetLastError();
}

cudaError_t launch_bucket_starts_fix(cudaStream_t st, const BucketParams& bp, uint32_t* start) {
    k_bkt_starts_fix<<<1, 1024, 0, st>>>(bp, start);
    return cudaGetLastError();
}

uint64_t bucket_tile_records() { return BK_TILE; }

template <int ST, bool IQ>
static cudaError_t apply_one(const TableParams& tp, const BucketParams& bp, const uint64_t* recs,
                             const uint32_t* start, uint32_t* new_bits,
                             unsigned long long* counters, uint8_t* vals, cudaStream_t st) {
    const size_t smem = bk_apply_smem((1u << bp.fs) / cells_per_word<ST>(), IQ);
    cudaError_t e = cudaFuncSetAttribute(k_bkt_apply<ST, IQ>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bkt_apply<ST, IQ><<<bp.n_buckets, BK_BLOCK, smem, st>>>(tp, bp, recs, start, new_bits,
                                                              counters, vals);
    return cudaGetLastError();
}

cudaError_t launch_bucket_apply(int storage, const TableParams& tp, const BucketParams& bp,
                                const uint64_t* recs, const uint32_t* start, uint32_t* new_bits,
                                unsigned long long* counters, uint8_t* vals, cudaStream_t st) {
    if (bp.n_buckets == 0) return cudaSuccess;
    switch (storage) {
    case GDBG_BIT: return apply_one<GDBG_BIT, false>(tp, bp, recs, start, new_bits, counters, nullptr, st);
    case GDBG_BYTE:
        return vals ? apply_one<GDBG_BYTE, true>(tp, bp, recs, start, new_bits, counters, vals, st)
                    : apply_one<GDBG_BYTE, false>(tp, bp, recs, start, new_bits, counters, nullptr, st);
    default:
        return vals ? apply_one<GDBG_NIBBLE, true>(tp, bp, recs, start, new_bits, counters, vals, st)
                    : apply_one<GDBG_NIBBLE, false>(tp, bp, recs, start, new_bits, counters, nullptr, st);
    }
}

cudaError_t launch_iq_counts(const uint8_t* vals, uint64_t cap, uint32_t n_tables,
                             const uint32_t* new_bits, const uint64_t* total, int16_t* counts,
                             bool presence, cudaStream_t st) {
    if (cap == 0) return cudaSuccess;
    uint64_t grid = (cap + 255) / 256;
    if (grid > 152 * 16) grid = 152 * 16;
    k_iq_counts<<<(unsigned)grid, 256, 0, st>>>(vals, cap, n_tables, new_bits, total, counts, presence);
    return cudaGetLastError();
}

cudaError_t launch_bucket_read_new(const uint64_t* kofs, uint64_t n_reads, const uint32_t* new_bits,
                                   uint64_t* n_new, unsigned long long* counters, cudaStream_t st) {
    if (n_reads == 0) return cudaSuccess;
    k_bkt_read_new<<<(unsigned)((n_reads + 255) / 256), 256, 0, st>>>(
        kofs, n_reads, new_bits, (unsigned long long*)n_new, counters);
    return cudaGetLastError();
}

// ---- exclusive scan of uint32 (histograms) --------------------------------
constexpr int SCAN32_BLOCK = 1024;
constexpr int SCAN32_ITEMS = 4;   // per thread

__device__ __forceinline__ uint32_t block_scan32(uint32_t v, uint32_t* ws) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) ws[wid] = v;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += t;
        }
        ws[lane] = s;
    }
    __syncthreads();
    if (wid > 0) v += ws[wid - 1];
    __syncthreads();
    return v;
}

// Both kernels take chunks c = blockIdx.x, blockIdx.x + gridDim.x, ... of
// SCAN32_BLOCK * SCAN32_ITEMS entries (a gated scan launches a small grid,
// so it costs little when the gate keeps it idle).
__global__ void __launch_bounds__(SCAN32_BLOCK)
k_scan32_partials(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ partials,
                  const uint32_t* gate, uint64_t n_chunks) {
    __shared__ uint32_t ws[32];
    if (gate && *(volatile const uint32_t*)gate == 0) return;
    for (uint64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const uint64_t base = (c * SCAN32_BLOCK + threadIdx.x) * SCAN32_ITEMS;
        uint32_t s = 0;
#pragma unroll
        for (int j = 0; j < SCAN32_ITEMS; ++j)
            if (base + j < n) s += in[base + j];
        s = block_scan32(s, ws);
        if (threadIdx.x == SCAN32_BLOCK - 1) partials[c] = s;
    }
}

// Each block first sums the totals of the blocks before it (a few thousand at
// most), so no separate pass scans the partials.
__global__ void __launch_bounds__(SCAN32_BLOCK)
k_scan32_final(const uint32_t* __restrict__ in, uint64_t n, const uint32_t* __restrict__ partials,
               uint32_t* __restrict__ out, const uint32_t* gate, uint64_t n_chunks) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t before_s;
    if (gate && *(volatile const uint32_t*)gate == 0) return;
    for (uint64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        uint32_t pre = 0;
        for (uint64_t i = threadIdx.x; i < c; i += SCAN32_BLOCK) pre += partials[i];
        pre = block_scan32(pre, ws);
        if (threadIdx.x == SCAN32_BLOCK - 1) before_s = pre;
        __syncthreads();
        const uint32_t before = before_s;
        const uint64_t base = (c * SCAN32_BLOCK + threadIdx.x) * SCAN32_ITEMS;
        uint32_t v[SCAN32_ITEMS], s = 0;
#pragma unroll
        for (int j = 0; j < SCAN32_ITEMS; ++j) {
            v[j] = base + j < n ? in[base + j] : 0;
            s += v[j];
        }
        uint32_t run = block_scan32(s, ws) - s + before;
#pragma unroll
        for (int j = 0; j < SCAN32_ITEMS; ++j) {
            if (base + j < n) out[base + j] = run;
            run += v[j];
        }
        __syncthreads();   // before_s is rewritten for the next chunk
    }
}

uint64_t scan32_partials_needed(uint64_t n) {
    return (n + SCAN32_BLOCK * SCAN32_ITEMS - 1) / (SCAN32_BLOCK * SCAN32_ITEMS) + 1;
}

cudaError_t launch_scan32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* partials,
                          cudaStream_t st, const uint32_t* gate) {
    if (n == 0) return cudaSuccess;
    const uint64_t nb = (n + SCAN32_BLOCK * SCAN32_ITEMS - 1) / (SCAN32_BLOCK * SCAN32_ITEMS);
    uint64_t grid = nb;
    if (gate) {
        int dev = 0, sms = 152;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = std::min<uint64_t>(nb, 2 * (uint64_t)sms);
    }
    k_scan32_partials<<<(unsigned)grid, SCAN32_BLOCK, 0, st>>>(in, n, partials, gate, nb);
    k_scan32_final<<<(unsigned)grid, SCAN32_BLOCK, 0, st>>>(in, n, partials, out, gate, nb);
    return cudaGetLastError();
}

}  // namespace gdbg
