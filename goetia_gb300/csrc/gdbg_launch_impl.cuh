// Launcher definitions, instantiated once per storage kind by
// gdbg_kernels_{bit,byte,nibble}.cu.
#pragma once
#include "gdbg_kernels.cuh"
#include "gdbg_launch.h"
#include "gdbg_persist.cuh"

namespace gdbg {

inline unsigned grid_for(uint64_t n_threads) {
    return (unsigned)((n_threads + BLOCK - 1) / BLOCK);
}

template <int ST, bool C, int H, int NT, bool FH>
cudaError_t insert_pass_one(int pass, uint64_t n_threads, cudaStream_t st, const BatchView& b,
                            const uint64_t* hashes, const HashParams& hp, const TableParams& tp,
                            const WindowParams& w) {
    if (n_threads == 0) return cudaSuccess;
    if (pass == 0)
        k_probe<ST, C, H, NT, FH><<<grid_for(n_threads), BLOCK, 0, st>>>(b, hashes, hp, tp, w);
    else if (pass == 1)
        k_commit<ST, C, H, NT, FH><<<grid_for(n_threads), BLOCK, 0, st>>>(b, hashes, hp, tp, w);
    else if (n_threads <= (uint64_t)SMALL_BLOCK)
        k_insert_small<ST, C, H, NT, FH><<<1, SMALL_BLOCK, 0, st>>>(b, hashes, hp, tp, w);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// Probe and commit of at most SMALL_BLOCK k-mers in one block, one k-mer per
// thread: each thread's chain of dependent table updates is one k-mer long.
template <int ST, bool C, int NT, bool FH>
cudaError_t insert_small_one(uint64_t n_kmers, cudaStream_t st, const BatchView& b,
                             const uint64_t* hashes, const HashParams& hp, const TableParams& tp,
                             const WindowParams& w) {
    if (n_kmers == 0) return cudaSuccess;
    if (n_kmers > (uint64_t)SMALL_BLOCK) return cudaErrorInvalidValue;
    k_insert_small<ST, C, 1, NT, FH><<<1, SMALL_BLOCK, 0, st>>>(b, hashes, hp, tp, w);
    return cudaGetLastError();
}

template <int ST>
cudaError_t launch_insert_pass(int pass, const LaunchShape& s, uint64_t n_threads,
                               cudaStream_t st, const BatchView& b, const uint64_t* hashes,
                               const HashParams& hp, const TableParams& tp,
                               const WindowParams& w) {
    const bool fh = hashes != nullptr;
    const bool t4 = s.n_tables == 4;
    if (pass == 3) {   // n_threads = k-mers of the window
        if (fh)
            return t4 ? insert_small_one<ST, false, 4, true>(n_threads, st, b, hashes, hp, tp, w)
                      : insert_small_one<ST, false, 0, true>(n_threads, st, b, hashes, hp, tp, w);
        if (s.canonical)
            return t4 ? insert_small_one<ST, true, 4, false>(n_threads, st, b, hashes, hp, tp, w)
                      : insert_small_one<ST, true, 0, false>(n_threads, st, b, hashes, hp, tp, w);
        return t4 ? insert_small_one<ST, false, 4, false>(n_threads, st, b, hashes, hp, tp, w)
                  : insert_small_one<ST, false, 0, false>(n_threads, st, b, hashes, hp, tp, w);
    }
#define GDBG_PASS(C, H, NT, FH)                                                              \
    if (s.canonical == C && s.kmers_per_thread == H && (NT == 4) == t4 && fh == FH)          \
        return insert_pass_one<ST, C, H, NT, FH>(pass, n_threads, st, b, hashes, hp, tp, w);
    GDBG_PASS(true, 4, 4, false) GDBG_PASS(true, 8, 4, false)
    GDBG_PASS(false, 4, 4, false) GDBG_PASS(false, 8, 4, false)
    GDBG_PASS(true, 4, 0, false) GDBG_PASS(true, 8, 0, false)
    GDBG_PASS(false, 4, 0, false) GDBG_PASS(false, 8, 0, false)
    if (fh) {
        if (t4) return insert_pass_one<ST, false, 4, 4, true>(pass, n_threads, st, b, hashes, hp, tp, w);
        return insert_pass_one<ST, false, 4, 0, true>(pass, n_threads, st, b, hashes, hp, tp, w);
    }
#undef GDBG_PASS
    return cudaErrorInvalidValue;
}

template <int ST, bool C, int NT, bool FH>
cudaError_t query_one(uint64_t n_total, cudaStream_t st, const BatchView& b, const uint64_t* hashes,
                      const HashParams& hp, const TableParams& tp, int16_t* counts,
                      uint64_t* values) {
    constexpr int H = 4;
    uint64_t n_threads = (n_total + H - 1) / H;
    if (n_threads == 0) return cudaSuccess;
    k_query<ST, C, H, NT, FH><<<grid_for(n_threads), BLOCK, 0, st>>>(b, hashes, hp, tp, n_total,
                                                                     counts, values);
    return cudaGetLastError();
}

template <int ST>
cudaError_t launch_query(const LaunchShape& s, uint64_t n_total, cudaStream_t st,
                         const BatchView& b, const uint64_t* hashes, const HashParams& hp,
                         const TableParams& tp, int16_t* counts, uint64_t* values) {
    const bool t4 = s.n_tables == 4;
    if (hashes) {
        if (t4) return query_one<ST, false, 4, true>(n_total, st, b, hashes, hp, tp, counts, values);
        return query_one<ST, false, 0, true>(n_total, st, b, hashes, hp, tp, counts, values);
    }
    if (s.canonical) {
        if (t4) return query_one<ST, true, 4, false>(n_total, st, b, hashes, hp, tp, counts, values);
        return query_one<ST, true, 0, false>(n_total, st, b, hashes, hp, tp, counts, values);
    }
    if (t4) return query_one<ST, false, 4, false>(n_total, st, b, hashes, hp, tp, counts, values);
    return query_one<ST, false, 0, false>(n_total, st, b, hashes, hp, tp, counts, values);
}

template <int ST, bool C, int NT>
cudaError_t masks_one(cudaStream_t st, const BatchView& b, const HashParams& hp,
                      const TableParams& tp, uint8_t* masks) {
    constexpr int H = 2;
    uint64_t n_threads = (b.n_kmers + H - 1) / H;
    if (n_threads == 0) return cudaSuccess;
    bool small = NT == 4;   // the generic table count keeps 64-bit remainders
    for (int i = 0; i < tp.n; ++i) small = small && tp.p[i] < (1ull << 31);
    if (small) k_masks<ST, C, H, NT, true><<<grid_for(n_threads), BLOCK, 0, st>>>(b, hp, tp, masks);
    else k_masks<ST, C, H, NT, false><<<grid_for(n_threads), BLOCK, 0, st>>>(b, hp, tp, masks);
    return cudaGetLastError();
}

template <int ST>
cudaError_t launch_masks(const LaunchShape& s, cudaStream_t st, const BatchView& b,
                         const HashParams& hp, const TableParams& tp, uint8_t* masks) {
    const bool t4 = s.n_tables == 4;
    if (s.canonical) return t4 ? masks_one<ST, true, 4>(st, b, hp, tp, masks)
                               : masks_one<ST, true, 0>(st, b, hp, tp, masks);
    return t4 ? masks_one<ST, false, 4>(st, b, hp, tp, masks)
              : masks_one<ST, false, 0>(st, b, hp, tp, masks);
}

template <int ST, bool C, int NT>
cudaError_t persist_one(uint64_t max_tasks, cudaStream_t st, const BatchView& b,
                        const HashParams& hp, const TableParams& tp, const PersistParams& pp,
                        int* grid_used) {
    auto kern = k_insert_persistent<ST, C, NT>;
    // co-resident blocks of the current device (occupancy queries are cheap
    // and per device, so nothing is cached across calls or devices)
    int dev = 0, n_sm = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PBLOCK, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1 || n_sm < 1) return cudaErrorInvalidConfiguration;
    uint64_t want = (max_tasks * 32 + PBLOCK - 1) / PBLOCK;
    uint64_t grid = (uint64_t)per_sm * n_sm;
    if (want < grid) grid = want ? want : 1;
    *grid_used = (int)grid;
    BatchView b_ = b;
    HashParams hp_ = hp;
    TableParams tp_ = tp;
    PersistParams pp_ = pp;
    void* args[] = {&b_, &hp_, &tp_, &pp_};
    return cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)grid), dim3(PBLOCK), args,
                                       0, st);
}

template <int ST>
cudaError_t launch_insert_persistent(const LaunchShape& s, uint64_t max_tasks, cudaStream_t st,
                                     const BatchView& b, const HashParams& hp,
                                     const TableParams& tp, const PersistParams& pp,
                                     int* grid_used) {
    const bool t4 = s.n_tables == 4;
    if (s.canonical) return t4 ? persist_one<ST, true, 4>(max_tasks, st, b, hp, tp, pp, grid_used)
                               : persist_one<ST, true, 0>(max_tasks, st, b, hp, tp, pp, grid_used);
    return t4 ? persist_one<ST, false, 4>(max_tasks, st, b, hp, tp, pp, grid_used)
              : persist_one<ST, false, 0>(max_tasks, st, b, hp, tp, pp, grid_used);
}

static_assert(READ_MAXNT == READ_INSERT_MAXNT, "one table limit for the read insert");

// One read in one CTA (k_insert_read): 48 KB of map beside the kernel's own
// shared words, so the launch opts in to more than the default 48 KB (once
// per handle: set_attr).
template <int ST>
cudaError_t launch_insert_read(bool canonical, bool set_attr, cudaStream_t st, const BatchView& b,
                               const HashParams& hp, const TableParams& tp, uint64_t* n_new,
                               unsigned long long* counters, uint32_t* err, uint64_t* done,
                               uint32_t seq) {
    if (tp.n > READ_MAXNT) return cudaErrorInvalidValue;
    const int smem = (int)read_insert_smem();
    auto go = [&](auto kern) {
        if (set_attr) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<1, READ_BLOCK, smem, st>>>(b, hp, tp, n_new, counters, err, done, seq);
        return cudaGetLastError();
    };
    // both forms' attributes on the first call, whichever shifter it uses
    if (set_attr) {
        cudaError_t e = cudaFuncSetAttribute(canonical ? k_insert_read<ST, false> : k_insert_read<ST, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    return canonical ? go(k_insert_read<ST, true>) : go(k_insert_read<ST, false>);
}

#define GDBG_INSTANTIATE_LAUNCHERS(ST)                                                         \
    template cudaError_t launch_insert_pass<ST>(int, const LaunchShape&, uint64_t, cudaStream_t, \
                                                const BatchView&, const uint64_t*,             \
                                                const HashParams&, const TableParams&,         \
                                                const WindowParams&);                          \
    template cudaError_t launch_query<ST>(const LaunchShape&, uint64_t, cudaStream_t,          \
                                          const BatchView&, const uint64_t*, const HashParams&, \
                                          const TableParams&, int16_t*, uint64_t*);            \
    template cudaError_t launch_masks<ST>(const LaunchShape&, cudaStream_t, const BatchView&,  \
                                          const HashParams&, const TableParams&, uint8_t*);    \
    template cudaError_t launch_insert_persistent<ST>(const LaunchShape&, uint64_t, cudaStream_t, \
                                                      const BatchView&, const HashParams&,    \
                                                      const TableParams&, const PersistParams&, \
                                                      int*);                                   \
    template cudaError_t launch_insert_read<ST>(bool, bool, cudaStream_t, const BatchView&,   \
                                                const HashParams&, const TableParams&, uint64_t*, \
                                                unsigned long long*, uint32_t*, uint64_t*, uint32_t);

}  // namespace gdbg
