// Launchers for the segmented bucketed insert (kernels in gdbg_sort.cuh).
#include <algorithm>

#include "gdbg_launch.h"
#include "gdbg_sort.cuh"
#include "gdbg_emit_part.cuh"

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

cudaError_t launch_sp_groups(cudaStream_t st, const SortParams& sp) {
    k_sp_groups<<<1, 256, 0, st>>>(sp);
    return cudaGetLastError();
}

cudaError_t launch_sp_emit_part(bool canonical, cudaStream_t st, const BatchView& b, const HashParams& hp,
                                const TableParams& tp, const SortParams& sp, uint64_t* rout,
                                uint32_t seg0, uint32_t n_seg) {
    if (n_seg == 0 || seg0 >= sp.nseg1) return cudaSuccess;
    if (n_seg > sp.nseg1 - seg0) n_seg = sp.nseg1 - seg0;
    bool small = true;   // every table below 2^31 cells: 32-bit remainders
    for (int i = 0; i < tp.n; ++i) small = small && tp.p[i] < (1ull << 31);
    const size_t smem = sp_ep_smem();
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<n_seg, SP_EP_BLOCK, smem, st>>>(b, hp, tp, sp, rout, seg0);
        return cudaGetLastError();
    };
    if (canonical) return small ? go(k_sp_emit_part<true, true>) : go(k_sp_emit_part<true, false>);
    return small ? go(k_sp_emit_part<false, true>) : go(k_sp_emit_part<false, false>);
}

template <bool PASS2, bool RESERVE>
static cudaError_t sp_part_one(cudaStream_t st, const SortParams& sp, uint32_t grid, const uint64_t* rin,
                               uint64_t* rout) {
    const size_t smem = sp_part_smem();
    cudaError_t e = cudaFuncSetAttribute(k_sp_part<PASS2, RESERVE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_sp_part<PASS2, RESERVE><<<grid, SP_PART_BLOCK, smem, st>>>(sp, rin, rout);
    return cudaGetLastError();
}

static uint32_t sm_count() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (uint32_t)sms;
}

// Pass 1 and the reserved pass 2 take one segment per CTA; the counted pass
// 2 and a gated pass 1, which usually return at once, loop over the segments
// with two CTAs per SM (as many as fit), so their launches cost little when
// they have no work.
cudaError_t launch_sp_part(int pass, cudaStream_t st, const SortParams& sp, const uint64_t* rin,
                           uint64_t* rout) {
    uint32_t grid = pass == SP_PASS1 ? sp.nseg1 : sp.nseg2_cap;
    if (grid == 0) return cudaSuccess;
    if (pass == SP_PASS2_COUNTED || (pass == SP_PASS1 && sp.gate1)) grid = std::min(grid, 2 * sm_count());
    switch (pass) {
    case SP_PASS1: return sp_part_one<false, false>(st, sp, grid, rin, rout);
    case SP_PASS2_RESERVED: return sp_part_one<true, true>(st, sp, grid, rin, rout);
    default: return sp_part_one<true, false>(st, sp, grid, rin, rout);
    }
}

cudaError_t launch_sp_plan(cudaStream_t st, const SortParams& sp) {
    k_sp_plan<<<1, 256, 0, st>>>(sp);
    return cudaGetLastError();
}

cudaError_t launch_sp_hist2(cudaStream_t st, const SortParams& sp, const uint64_t* rin) {
    if (sp.nseg2_cap == 0) return cudaSuccess;
    k_sp_hist2<<<std::min(sp.nseg2_cap, 4 * sm_count()), SP_PART_BLOCK, 0, st>>>(sp, rin);
    return cudaGetLastError();
}

cudaError_t launch_sp_starts(cudaStream_t st, const SortParams& sp, uint32_t* start, uint32_t* end) {
    const uint32_t n = sp.n_buckets;
    if (n == 0) return cudaSuccess;
    k_sp_starts<<<(n + 255) / 256, 256, 0, st>>>(sp, start, end);
    return cudaGetLastError();
}

// Map slots of the apply for regions of region_words words: the shared
// memory that SP_APPLY_CTAS CTAs per SM leave beside their regions (fewer
// CTAs when that leaves under 1024 slots, for the largest regions), at most
// 8192 slots (10 bytes each: the entry and its place on the created list).
static uint32_t sp_map_slots(uint32_t region_words) {
    int dev = 0, per_sm = 228 * 1024, reserved = 1024;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    }
    const size_t static_b = 256;   // the kernel's own __shared__ words, rounded up
    const size_t fixed = sp_apply_smem(region_words, 0) + static_b + (size_t)reserved;
    uint32_t slots = 0;
    for (int ctas = SP_APPLY_CTAS; ctas >= 1 && slots < 1024; --ctas) {
        const size_t per = (size_t)per_sm / ctas;
        slots = per > fixed + 16 ? (uint32_t)std::min<size_t>((per - fixed - 16) / 10, 8192) : 0u;
    }
    return slots & ~31u;
}

template <int ST>
static cudaError_t sp_apply_one(const TableParams& tp, const SortParams& sp_in, const uint64_t* recs,
                                const uint32_t* start, const uint32_t* end, uint32_t* new_bits,
                                unsigned long long* counters, cudaStream_t st) {
    SortParams sp = sp_in;
    const uint32_t region_words = (1u << sp.fs) / cells_per_word<ST>();
    sp.map_slots = sp_map_slots(region_words);
    if (sp.map_slots == 0) return cudaErrorInvalidConfiguration;
    const size_t smem = sp_apply_smem(region_words, sp.map_slots);
    cudaError_t e = cudaFuncSetAttribute(k_sp_apply<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_sp_apply<ST><<<sp.n_buckets, SP_APPLY_BLOCK, smem, st>>>(tp, sp, recs, start, end, new_bits, counters);
    return cudaGetLastError();
}

cudaError_t launch_sp_apply(int storage, const TableParams& tp, const SortParams& sp,
                            const uint64_t* recs, const uint32_t* start, const uint32_t* end,
                            uint32_t* new_bits, unsigned long long* counters, cudaStream_t st) {
    if (sp.n_buckets == 0) return cudaSuccess;
    switch (storage) {
    case GDBG_BIT: return sp_apply_one<GDBG_BIT>(tp, sp, recs, start, end, new_bits, counters, st);
    case GDBG_BYTE: return sp_apply_one<GDBG_BYTE>(tp, sp, recs, start, end, new_bits, counters, st);
    default: return sp_apply_one<GDBG_NIBBLE>(tp, sp, recs, start, end, new_bits, counters, st);
    }
}

size_t sp_apply_smem_bytes(int storage, uint32_t fs) {
    const uint32_t cpw = storage == GDBG_BIT ? 32u : storage == GDBG_BYTE ? 4u : 8u;
    const uint32_t region_words = (1u << fs) / cpw;
    return sp_apply_smem(region_words, sp_map_slots(region_words));
}

}  // namespace gdbg
