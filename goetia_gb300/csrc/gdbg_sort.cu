// Launchers for the segmented bucketed insert (kernels in gdbg_sort.cuh).
#include <algorithm>
#include <cmath>

#include "gdbg_launch.h"
#include "gdbg_sort.cuh"

namespace gdbg {

cudaError_t launch_sp_emit(bool canonical, cudaStream_t st, const BatchView& b, const HashParams& hp,
                           const TableParams& tp, const SortParams& sp, uint64_t* rout,
                           uint32_t seg0, uint32_t n_seg) {
    if (n_seg == 0 || seg0 >= sp.nseg1) return cudaSuccess;
    if (n_seg > sp.nseg1 - seg0) n_seg = sp.nseg1 - seg0;
    const bool t4 = sp.n_tables == 4;
    bool small = true;   // every table below 2^31 cells: 32-bit remainders
    for (int i = 0; i < tp.n; ++i) small = small && tp.p[i] < (1ull << 31);
    const unsigned g = n_seg;
#define GDBG_EMIT(C, N, S) k_sp_emit<C, N, S><<<g, SP_EMIT_BLOCK, 0, st>>>(b, hp, tp, sp, rout, seg0)
    if (canonical) {
        if (t4) small ? GDBG_EMIT(true, 4, true) : GDBG_EMIT(true, 4, false);
        else small ? GDBG_EMIT(true, 0, true) : GDBG_EMIT(true, 0, false);
    } else {
        if (t4) small ? GDBG_EMIT(false, 4, true) : GDBG_EMIT(false, 4, false);
        else small ? GDBG_EMIT(false, 0, true) : GDBG_EMIT(false, 0, false);
    }
#undef GDBG_EMIT
    return cudaGetLastError();
}

cudaError_t launch_sp_part(bool pass2, cudaStream_t st, const SortParams& sp, const uint64_t* rin,
                           uint64_t* rout) {
    const uint32_t grid = pass2 ? sp.nseg2_cap : sp.nseg1;
    if (grid == 0) return cudaSuccess;
    const size_t smem = sp_part_smem();
    cudaError_t e;
    if (pass2) {
        e = cudaFuncSetAttribute(k_sp_part<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_sp_part<true><<<grid, SP_PART_BLOCK, smem, st>>>(sp, rin, rout);
    } else {
        e = cudaFuncSetAttribute(k_sp_part<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_sp_part<false><<<grid, SP_PART_BLOCK, smem, st>>>(sp, rin, rout);
    }
    return cudaGetLastError();
}

cudaError_t launch_sp_plan(cudaStream_t st, const SortParams& sp) {
    k_sp_plan<<<1, 256, 0, st>>>(sp);
    return cudaGetLastError();
}

cudaError_t launch_sp_hist2(cudaStream_t st, const SortParams& sp, const uint64_t* rin) {
    if (sp.nseg2_cap == 0) return cudaSuccess;
    k_sp_hist2<<<sp.nseg2_cap, SP_PART_BLOCK, 0, st>>>(sp, rin);
    return cudaGetLastError();
}

cudaError_t launch_sp_starts(cudaStream_t st, const SortParams& sp, uint32_t* start) {
    const uint32_t n = sp.n_buckets + 1;
    k_sp_starts<<<(n + 255) / 256, 256, 0, st>>>(sp, start);
    return cudaGetLastError();
}

// Shared-memory plan of the apply for regions of region_words words and
// buckets of about `load` records: the record buffer holds the load plus
// eight standard deviations of a Poisson count (4096 to 8192 records,
// indexable in the 32 - fs bits a map entry leaves; a rarer, fuller bucket
// takes the chunked path), and the map space is 16 KB when that keeps as
// many CTAs per SM (at most four of 512 threads) as 8 KB does.
struct ApplyPlan {
    uint32_t map_bytes, rbuf_cap, idx_bits;
};
static ApplyPlan sp_apply_plan(uint32_t region_words, uint32_t fs, double load) {
    int dev = 0, per_sm = 228 * 1024, reserved = 1024;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    }
    ApplyPlan p{};
    // cell << idx_bits | index stays below the all-ones empty entry (the
    // segmented path's regions are at most 64 KB, so fs <= 19)
    p.idx_bits = fs <= 18 ? 13u : 12u;
    const uint32_t cap_max = std::min<uint32_t>(SP_RBUF_MAX, 1u << p.idx_bits);
    const double want = load + 8.0 * std::sqrt(load) + 64.0;
    uint32_t rb = want >= cap_max ? cap_max : ((uint32_t)want + 63u) / 64u * 64u;
    p.rbuf_cap = std::min(std::max(rb, std::min(SP_RBUF_MIN, cap_max)), cap_max);
    const size_t static_b = 1024;   // the kernel's own __shared__ words, rounded up
    auto ctas = [&](uint32_t map_b) {
        const size_t per = sp_apply_smem(region_words, map_b, p.rbuf_cap) + static_b + (size_t)reserved;
        return (int)std::min<size_t>(4, (size_t)per_sm / per);
    };
    p.map_bytes = ctas(SP_MAP_MAX) >= ctas(SP_MAP_MIN) ? SP_MAP_MAX : SP_MAP_MIN;
    return p;
}

// Expected records per bucket of the batch: its k-mer bound times the cells
// of a bucket over the smallest table.
static double sp_bucket_load(const TableParams& tp, const SortParams& sp) {
    uint64_t pmin = ~0ull;
    for (int i = 0; i < tp.n; ++i) pmin = std::min<uint64_t>(pmin, tp.p[i]);
    return (double)sp.kmer_cap * (double)(1ull << sp.fs) / (double)pmin;
}

template <int ST>
static cudaError_t sp_apply_one(const TableParams& tp, const SortParams& sp_in, const uint64_t* recs,
                                const uint32_t* start, uint32_t* new_bits,
                                unsigned long long* counters, cudaStream_t st) {
    SortParams sp = sp_in;
    const uint32_t region_words = (1u << sp.fs) / cells_per_word<ST>();
    const ApplyPlan plan = sp_apply_plan(region_words, sp.fs, sp_bucket_load(tp, sp));
    sp.map_bytes = plan.map_bytes;
    sp.rbuf_cap = plan.rbuf_cap;
    sp.idx_bits = plan.idx_bits;
    const size_t smem = sp_apply_smem(region_words, sp.map_bytes, sp.rbuf_cap);
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<sp.n_buckets, SP_APPLY_BLOCK, smem, st>>>(tp, sp, recs, start, new_bits, counters);
        return cudaGetLastError();
    };
    const bool big = sp.map_bytes == SP_MAP_MAX;
    if (sp.idx_bits == 13)
        return big ? go(k_sp_apply<ST, SP_MAP_MAX, 13>) : go(k_sp_apply<ST, SP_MAP_MIN, 13>);
    return big ? go(k_sp_apply<ST, SP_MAP_MAX, 12>) : go(k_sp_apply<ST, SP_MAP_MIN, 12>);
}

cudaError_t launch_sp_apply(int storage, const TableParams& tp, const SortParams& sp,
                            const uint64_t* recs, const uint32_t* start, uint32_t* new_bits,
                            unsigned long long* counters, cudaStream_t st) {
    if (sp.n_buckets == 0) return cudaSuccess;
    switch (storage) {
    case GDBG_BIT: return sp_apply_one<GDBG_BIT>(tp, sp, recs, start, new_bits, counters, st);
    case GDBG_BYTE: return sp_apply_one<GDBG_BYTE>(tp, sp, recs, start, new_bits, counters, st);
    default: return sp_apply_one<GDBG_NIBBLE>(tp, sp, recs, start, new_bits, counters, st);
    }
}

size_t sp_apply_smem_bytes(int storage, uint32_t fs) {
    const uint32_t cpw = storage == GDBG_BIT ? 32u : storage == GDBG_BYTE ? 4u : 8u;
    const ApplyPlan p = sp_apply_plan((1u << fs) / cpw, fs, SP_RBUF_MIN);
    return sp_apply_smem((1u << fs) / cpw, p.map_bytes, p.rbuf_cap);
}

}  // namespace gdbg
