// Compactor query of read batches (find_new_segments, compactor.hh:346-466):
// for every k-mer of a read, against the storage as it is,
//   flags bit 0  new  -- query() == 0
//   flags bit 1  seen -- its hash is already in the read's new-k-mer set
//                        (an earlier new k-mer of the same read has it)
//   mask         the 8 neighbours (hashextender.hh:352-396), each present
//                when query() != 0 or it is one of the read's new k-mers
//                (filter_nodes with extras, unitig_walker.hh:457-469).
// Each read owns a region of an open-addressing table of its new k-mers'
// hashes, at slot 4 * kofs[r] + 2 * r with 2^floor(log2(4 * k-mers + 2))
// slots (load below one half), so reads never share slots; a slot keeps the
// smallest position of its hash.  The all-ones hash (the empty-slot marker)
// is kept per read in a separate word.
#include "gdbg_kernels.cuh"
#include "gdbg_launch.h"

namespace gdbg {

constexpr uint64_t CQ_EMPTY = ~0ull;

struct CompactorParams {
    uint64_t* keys;       // per read region, CQ_EMPTY = free
    uint32_t* minpos;     // smallest position of the slot's hash in the read
    uint32_t* allones;    // per read: smallest position of the all-ones hash
    uint8_t* flags;
    uint8_t* masks;
    uint32_t* err;
};

struct CqRegion {
    uint64_t base;
    uint64_t mask;   // slots - 1
};

__device__ __forceinline__ CqRegion cq_region(const BatchView& b, uint64_t r) {
    const uint64_t kr = __ldg(b.kofs + r), nk = __ldg(b.kofs + r + 1) - kr;
    const uint64_t room = 4 * nk + 2;
    const uint64_t slots = 1ull << (63 - __clzll((long long)room));
    return CqRegion{4 * kr + 2 * r, slots - 1};
}

__device__ __forceinline__ uint64_t cq_home(uint64_t h) { return (h * 0x9E3779B97F4A7C15ull) >> 24; }

// Slot holding h in the read's region, or ~0 when absent.
__device__ __forceinline__ uint64_t cq_find(const CompactorParams& cp, const CqRegion& rg,
                                           uint64_t h) {
    uint64_t sl = cq_home(h) & rg.mask;
    for (uint64_t it = 0; it <= rg.mask; ++it) {
        const uint64_t cur = __ldcg(cp.keys + rg.base + sl);
        if (cur == CQ_EMPTY) return ~0ull;
        if (cur == h) return rg.base + sl;
        sl = (sl + 1) & rg.mask;
    }
    return ~0ull;
}

template <int STORAGE, bool CANON, int H, int NT>
__global__ void __launch_bounds__(BLOCK)
k_cq_new(BatchView b, HashParams hp, TableParams tp, CompactorParams cp) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = tid * H;
    Run<H> run;
    make_run<CANON, H, false>(b, hp, g0, b.n_kmers, run);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (!((run.valid >> j) & 1u)) continue;
        const uint64_t g = g0 + j, r = run.read[j], h = run.h[j];
        const bool is_new = !present<STORAGE, CANON, NT>(tp, h);
        cp.flags[g] = is_new ? 1 : 0;
        if (!is_new) continue;
        const uint32_t p = (uint32_t)(g - __ldg(b.kofs + r));
        if (h == CQ_EMPTY) {
            atomicMin(cp.allones + r, p);
            continue;
        }
        const CqRegion rg = cq_region(b, r);
        uint64_t sl = cq_home(h) & rg.mask;
        bool placed = false;
        for (uint64_t it = 0; it <= rg.mask; ++it) {
            unsigned long long* key = (unsigned long long*)(cp.keys + rg.base + sl);
            uint64_t cur = __ldcg(cp.keys + rg.base + sl);
            if (cur == CQ_EMPTY) cur = atomicCAS(key, CQ_EMPTY, h);
            if (cur == CQ_EMPTY || cur == h) {
                atomicMin(cp.minpos + rg.base + sl, p);
                placed = true;
                break;
            }
            sl = (sl + 1) & rg.mask;
        }
        if (!placed) atomicOr(cp.err, GDBG_ERR_CLAIMS_FULL);
    }
}

template <int STORAGE, bool CANON, int H, int NT>
__global__ void __launch_bounds__(BLOCK)
k_cq_masks(BatchView b, HashParams hp, TableParams tp, CompactorParams cp) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = tid * H;
    Run<H> run;
    make_run<CANON, H, true>(b, hp, g0, b.n_kmers, run);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (!((run.valid >> j) & 1u)) continue;
        const uint64_t g = g0 + j, r = run.read[j];
        const CqRegion rg = cq_region(b, r);
        const uint32_t ones = __ldcg(cp.allones + r);
        auto in_read = [&](uint64_t x) {
            return x == CQ_EMPTY ? ones != 0xFFFFFFFFu : cq_find(cp, rg, x) != ~0ull;
        };
        // seen: the read has the same new hash at an earlier position
        uint8_t f = cp.flags[g];
        if (f & 1u) {
            const uint32_t p = (uint32_t)(g - __ldg(b.kofs + r));
            const uint64_t h = run.h[j];
            const uint32_t first = h == CQ_EMPTY ? ones : __ldcg(cp.minpos + cq_find(cp, rg, h));
            if (first < p) f |= 2u;
            cp.flags[g] = f;
        }
        const uint64_t fw = run.fw[j], rc = run.rc[j];
        const uint32_t fr = run.front[j], bk = run.back[j];
        uint32_t m = 0;
#pragma unroll
        for (uint32_t c = 0; c < 4; ++c) {
            uint64_t lf = fw, lr = rc;
            roll_left<CANON>(hp, c, bk, lf, lr);
            const uint64_t lh = hash_value<CANON>(lf, lr);
            if (present<STORAGE, CANON, NT>(tp, lh) || in_read(lh)) m |= 1u << c;
            uint64_t rf = fw, rr = rc;
            roll_right<CANON>(hp, fr, c, rf, rr);
            const uint64_t rh = hash_value<CANON>(rf, rr);
            if (present<STORAGE, CANON, NT>(tp, rh) || in_read(rh)) m |= 1u << (4 + c);
        }
        cp.masks[g] = (uint8_t)m;
    }
}

template <int ST, bool C, int NT>
static cudaError_t cq_one(cudaStream_t st, const BatchView& b, const HashParams& hp,
                          const TableParams& tp, const CompactorParams& cp) {
    constexpr int H = 2;
    const uint64_t n_threads = (b.n_kmers + H - 1) / H;
    if (n_threads == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n_threads + BLOCK - 1) / BLOCK);
    k_cq_new<ST, C, H, NT><<<grid, BLOCK, 0, st>>>(b, hp, tp, cp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_cq_masks<ST, C, H, NT><<<grid, BLOCK, 0, st>>>(b, hp, tp, cp);
    return cudaGetLastError();
}

template <int ST>
static cudaError_t cq_storage(const LaunchShape& s, cudaStream_t st, const BatchView& b,
                              const HashParams& hp, const TableParams& tp,
                              const CompactorParams& cp) {
    const bool t4 = s.n_tables == 4;
    if (s.canonical) return t4 ? cq_one<ST, true, 4>(st, b, hp, tp, cp) : cq_one<ST, true, 0>(st, b, hp, tp, cp);
    return t4 ? cq_one<ST, false, 4>(st, b, hp, tp, cp) : cq_one<ST, false, 0>(st, b, hp, tp, cp);
}

cudaError_t launch_compactor(int storage, const LaunchShape& s, cudaStream_t st, const BatchView& b,
                             const HashParams& hp, const TableParams& tp, uint64_t* keys,
                             uint32_t* minpos, uint32_t* allones, uint8_t* flags, uint8_t* masks,
                             uint32_t* err) {
    const CompactorParams cp{keys, minpos, allones, flags, masks, err};
    switch (storage) {
    case GDBG_BIT: return cq_storage<GDBG_BIT>(s, st, b, hp, tp, cp);
    case GDBG_BYTE: return cq_storage<GDBG_BYTE>(s, st, b, hp, tp, cp);
    default: return cq_storage<GDBG_NIBBLE>(s, st, b, hp, tp, cp);
    }
}

uint64_t compactor_slots(uint64_t n_kmers, uint64_t n_reads) { return 4 * n_kmers + 2 * n_reads; }

}  // namespace gdbg
