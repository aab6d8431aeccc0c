// Device-side read packing: text reads already in device memory -> 2-bit
// packed stream + base offsets, with the FASTX policy of goetia's DNA_SIMPLE
// reader (FastxParser::next, include/goetia/parsing/readers.hh:150-219;
// Alphabet::validate, include/goetia/sequences/alphabets.hh:41-56,107-130):
// lowercase acgt are upper-cased, a read holding any other symbol or shorter
// than min_length is dropped and counted.  Same output as gdbg_pack_reads.
//
//   k_pk_check  one warp per read: validity and kept length
//   scans       kept bases and kept reads (exclusive, 32-bit)
//   k_pk_write  one warp per kept read, one lane per output word, codes by
//               arithmetic on the bytes (atomic OR for the words shared
//               with neighbour reads); the read's end offset
//   k_pk_final  counts and offsets[0]
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>

#include "gdbg_launch.h"
#include "goetia_gb300.h"

namespace gdbg {

constexpr int PK_BLOCK = 256;

// A DNA_SIMPLE symbol (ACGT, either case): (c | 0x20) - 'a' is 0, 2, 6 or 19
// exactly for them.
__device__ __forceinline__ bool pk_valid(unsigned char c) {
    const uint32_t d = (uint32_t)(c | 0x20u) - (uint32_t)'a';
    return d < 20u && ((0x80045u >> d) & 1u);
}

__global__ void __launch_bounds__(PK_BLOCK)
k_pk_check(const unsigned char* __restrict__ seqs, const uint64_t* __restrict__ starts,
           const uint64_t* __restrict__ ends, uint64_t n,
           uint32_t min_len, uint32_t* __restrict__ klen, uint32_t* __restrict__ kflag,
           uint32_t* err, uint32_t* both) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_warps = (uint64_t)gridDim.x * PK_BLOCK / 32;
    for (uint64_t r = ((uint64_t)blockIdx.x * PK_BLOCK + threadIdx.x) / 32; r < n; r += n_warps) {
        const uint64_t a = starts[r], b = ends[r];
        bool ok = b >= a && b - a < (1ull << 31);
        if (!ok && lane == 0) atomicOr(err, GDBG_ERR_BAD_OFFSETS);
        const uint64_t L = ok ? b - a : 0;
        for (uint64_t i = lane; i < L && ok; i += 32) ok = pk_valid(seqs[a + i]);
        ok = __all_sync(0xFFFFFFFFu, ok);
        const bool kept = ok && L >= min_len;
        if (lane == 0) {
            klen[r] = kept ? (uint32_t)L : 0u;
            kflag[r] = kept ? 1u : 0u;
            // FastxParser counts a read that is invalid and short twice
            if (both && !ok && L < min_len) atomicAdd(both, 1u);
        }
    }
}

// One warp per kept read, one lane per output word: lane l builds word
// w0 + l (+ 32, ...) from its (up to) 16 bases, each base's code by
// arithmetic on its byte -- ((c >> 1) & 3) gives A 0, C 1, G 3, T 2 for
// upper and lower case, and x ^ (x >> 1) swaps G and T (the reads here are
// valid: k_pk_check kept them).  A word that lies inside the read is
// stored; the read's first and last words, which neighbour reads share, are
// ORed in.
__global__ void __launch_bounds__(PK_BLOCK)
k_pk_write(const unsigned char* __restrict__ seqs, const uint64_t* __restrict__ starts, uint64_t n,
           const uint32_t* __restrict__ klen, const uint32_t* __restrict__ kflag,
           const uint32_t* __restrict__ kbase, const uint32_t* __restrict__ kidx,
           uint32_t* __restrict__ packed, uint64_t packed_words, uint64_t* __restrict__ offsets,
           uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_warps = (uint64_t)gridDim.x * PK_BLOCK / 32;
    for (uint64_t r = ((uint64_t)blockIdx.x * PK_BLOCK + threadIdx.x) / 32; r < n; r += n_warps) {
        if (!kflag[r]) continue;   // kept reads include empty ones (min_length 0)
        const uint64_t L = klen[r];
        const uint64_t a = starts[r], ob0 = kbase[r], ob1 = ob0 + L;
        if (L && (ob1 - 1) / 16 >= packed_words) {
            if (lane == 0) atomicOr(err, GDBG_ERR_BAD_OFFSETS);
            continue;
        }
        if (L) {
            const uint64_t w1 = (ob1 - 1) >> 4;
            for (uint64_t w = (ob0 >> 4) + lane; w <= w1; w += 32) {
                const uint64_t lo = w * 16 > ob0 ? w * 16 : ob0;
                const uint64_t hi = w * 16 + 16 < ob1 ? w * 16 + 16 : ob1;
                const unsigned char* src = seqs + a + (lo - ob0);
                const uint32_t q0 = (uint32_t)(lo & 15u), nb = (uint32_t)(hi - lo);
                uint32_t v = 0;
#pragma unroll
                for (uint32_t k = 0; k < 16; ++k) {
                    if (k < nb) {
                        const uint32_t x = ((uint32_t)src[k] >> 1) & 3u;
                        v |= (x ^ (x >> 1)) << (2u * (q0 + k));
                    }
                }
                if (nb == 16) packed[w] = v;
                else atomicOr(packed + w, v);
            }
        }
        if (lane == 0) offsets[(uint64_t)kidx[r] + 1] = ob1;
    }
}

__global__ void k_pk_final(const uint32_t* klen, const uint32_t* kbase, const uint32_t* kflag,
                           const uint32_t* kidx, uint64_t n, uint64_t* offsets, uint64_t* counts,
                           const uint32_t* both) {
    offsets[0] = 0;
    const uint64_t kept = n ? (uint64_t)kidx[n - 1] + kflag[n - 1] : 0;
    counts[0] = kept;
    counts[1] = n - kept;
    counts[2] = n ? (uint64_t)kbase[n - 1] + klen[n - 1] : 0;
    counts[3] = *both;
}

// Scratch of the packer and the FASTX parser comes from a pool of the
// library's own per device, which keeps up to SCRATCH_KEEP bytes between
// calls: the device's default pool gives its memory back at every
// synchronisation, and mapping a batch's scratch again costs more than the
// batch's kernels.  The pools live as long as the process.
constexpr uint64_t SCRATCH_KEEP = 2ull << 30;

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t st) {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = pools.find(dev);
        if (it == pools.end()) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
            uint64_t keep = SCRATCH_KEEP;
            if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
                return e;
            pools[dev] = pool;
        } else {
            pool = it->second;
        }
    }
    return cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, st);
}

// The packing of n_seqs text reads in device memory (read r =
// seqs[starts[r], ends[r])); out[0] kept, [1] dropped, [2] dropped reads
// that were both invalid and shorter than min_length.  Returns when done.
int pack_device_run(const char* seqs, const uint64_t* starts, const uint64_t* ends, uint64_t n_seqs,
                    uint32_t min_length, uint32_t* packed, uint64_t packed_words,
                    uint64_t* offsets, uint64_t out[3], cudaStream_t st) {
    if (n_seqs >= (1ull << 31)) return report_error(GDBG_ERR_INVALID_ARG, "too many reads for one call");
    const uint64_t parts = scan32_partials_needed(n_seqs + 1) + 1;
    // scratch: klen, kflag, kbase, kidx (n + 1 each), scan partials, err, both, counts
    const size_t bytes = (4 * (n_seqs + 1) + parts + 2) * sizeof(uint32_t) + 5 * sizeof(uint64_t);
    void* scratch = nullptr;
    cudaError_t e = scratch_alloc(&scratch, bytes, st);
    if (e != cudaSuccess) return report_error(GDBG_ERR_OOM, std::string("pack scratch: ") + cudaGetErrorString(e));
    uint32_t* klen = (uint32_t*)scratch;
    uint32_t* kflag = klen + (n_seqs + 1);
    uint32_t* kbase = kflag + (n_seqs + 1);
    uint32_t* kidx = kbase + (n_seqs + 1);
    uint32_t* partials = kidx + (n_seqs + 1);
    uint32_t* err = partials + parts;
    uint32_t* both = err + 1;
    uint64_t* counts = (uint64_t*)(((uintptr_t)(both + 1) + 7) & ~(uintptr_t)7);
    auto done = [&](int rc, const std::string& msg) {
        cudaFreeAsync(scratch, st);
        cudaStreamSynchronize(st);
        return rc == GDBG_OK ? rc : report_error(rc, msg);
    };
    if ((e = cudaMemsetAsync(err, 0, 2 * sizeof(uint32_t), st)) != cudaSuccess ||
        (packed_words && (e = cudaMemsetAsync(packed, 0, packed_words * sizeof(uint32_t), st)) != cudaSuccess))
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    uint64_t grid = (n_seqs * 32 + PK_BLOCK - 1) / PK_BLOCK;
    if (grid > 152 * 32) grid = 152 * 32;
    if (grid == 0) grid = 1;
    k_pk_check<<<(unsigned)grid, PK_BLOCK, 0, st>>>((const unsigned char*)seqs, starts, ends, n_seqs,
                                                    min_length, klen, kflag, err, both);
    if (n_seqs) {
        if ((e = launch_scan32(klen, kbase, n_seqs, partials, st)) != cudaSuccess ||
            (e = launch_scan32(kflag, kidx, n_seqs, partials, st)) != cudaSuccess)
            return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    }
    k_pk_write<<<(unsigned)grid, PK_BLOCK, 0, st>>>((const unsigned char*)seqs, starts, n_seqs,
                                                    klen, kflag, kbase, kidx, packed, packed_words,
                                                    offsets, err);
    k_pk_final<<<1, 1, 0, st>>>(klen, kbase, kflag, kidx, n_seqs, offsets, counts, both);
    if ((e = cudaGetLastError()) != cudaSuccess) return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    uint64_t hc[4] = {0, 0, 0, 0};
    uint32_t herr = 0;
    cudaMemcpyAsync(hc, counts, sizeof hc, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(scratch, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return report_error(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (herr) return report_error(GDBG_ERR_INVALID_ARG, "read offsets decrease, a read is 2^31 bases or longer, or packed is too small");
    out[0] = hc[0];
    out[1] = hc[1];
    out[2] = hc[3];
    return GDBG_OK;
}

}  // namespace gdbg

using namespace gdbg;

extern "C" int gdbg_pack_reads_device(const char* seqs, const uint64_t* seq_offsets, uint64_t n_seqs,
                                      uint32_t min_length, uint32_t* packed, uint64_t packed_words,
                                      uint64_t* offsets, uint64_t* n_kept, uint64_t* n_skipped,
                                      void* stream) {
    if (!seq_offsets || !offsets || !n_kept || !n_skipped || (!seqs && n_seqs) ||
        (!packed && packed_words))
        return report_error(GDBG_ERR_INVALID_ARG, "NULL argument");
    uint64_t out[3];
    const int rc = pack_device_run(seqs, seq_offsets, seq_offsets + 1, n_seqs, min_length, packed,
                                   packed_words, offsets, out, (cudaStream_t)stream);
    if (rc != GDBG_OK) return rc;
    *n_kept = out[0];
    *n_skipped = out[1];
    return GDBG_OK;
}
