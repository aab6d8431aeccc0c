// Whole-table kernels: the OR-merge behind BitStorage::update_from
// (bitstorage.cc:103-137).
//
// The merge streams both tables once (16-byte vectors, grid-stride over the
// handle's single table allocation: every table padded to 256 bytes, so the
// vector count is exact and the padding is zero in both operands).  The
// reference counts the cells that become occupied in table 0 as the popcount
// of (old ^ merged) per byte; here per 16-byte vector, the same sum.
#include "gdbg_launch.h"

namespace gdbg {

constexpr int MERGE_BLOCK = 256;

__global__ void __launch_bounds__(MERGE_BLOCK)
k_or_merge(uint4* __restrict__ dst, const uint4* __restrict__ src, uint64_t n_vec,
           uint64_t count_vec, unsigned long long* __restrict__ occupied) {
    unsigned long long added = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_vec; i += stride) {
        const uint4 a = dst[i], b = __ldg(src + i);
        const uint4 m = make_uint4(a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w);
        if (i < count_vec)
            added += __popc(a.x ^ m.x) + __popc(a.y ^ m.y) + __popc(a.z ^ m.z) + __popc(a.w ^ m.w);
        dst[i] = m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) added += __shfl_down_sync(0xFFFFFFFFu, added, o);
    if ((threadIdx.x & 31) == 0 && added) atomicAdd(occupied, added);
}

cudaError_t launch_or_merge(uint32_t* dst, const uint32_t* src, uint64_t n_words,
                            uint64_t count_words, unsigned long long* occupied, cudaStream_t st) {
    const uint64_t n_vec = n_words / 4;
    if (!n_vec) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (n_vec + MERGE_BLOCK - 1) / MERGE_BLOCK;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 152) * 8;
    if (blocks > cap) blocks = cap;
    k_or_merge<<<(unsigned)blocks, MERGE_BLOCK, 0, st>>>((uint4*)dst, (const uint4*)src, n_vec,
                                                          count_words / 4, occupied);
    return cudaGetLastError();
}

}  // namespace gdbg
