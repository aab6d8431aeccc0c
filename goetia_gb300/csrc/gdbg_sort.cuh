// Segmented bucketed insert: the batch's random table updates as streams,
// with partition passes that need no stable ranking.
//
//   1. k_sp_emit: one block per segment of SP_SEGK k-mers hashes them (each
//      thread rolls along a run of consecutive k-mers) and writes one record
//      per table per k-mer, (global cell << 32) | k-mer ordinal, into the
//      segment's slots; it also counts the records' first digit
//      (bucket >> hi_shift) per segment.
//   2. k_sp_part<false>: one CTA per segment moves its records to their
//      digit groups.  Tiles of SP_TILE records stream into shared memory
//      with cp.async.bulk (two buffers in flight, mbarrier-tracked); ranks
//      inside a tile come from shared-memory atomics (any order), and each
//      bin's run is written contiguously at the segment's cursor.
//   3. k_sp_plan / k_sp_hist2 / k_sp_part<true>: every digit group is cut
//      into segments of SP_SEG2 records that never cross a group, counted by
//      the low digit and partitioned again; the scan is laid out group by
//      group, so its entries are final record positions and bucket starts.
//   4. k_sp_apply: one CTA per bucket loads its table region and records
//      into shared memory.  The records of a bucket are in no particular
//      order, so the first toucher of a cell is found as the minimum k-mer
//      ordinal over all the bucket's records: pass 1 puts every cell that is
//      zero in the region into a shared-memory map keyed by cell, holding
//      the minimum ordinal; pass 2 applies every record and flags the map's
//      minimum as new.  A region whose zero cells overflow the map is done
//      in narrower cell ranges.  That is the reference's sequential rule
//      (bitstorage.hh:195-219, bytestorage.cc:60-113, nibblestorage.cc:
//      60-100) cell by cell; a cell's final value does not depend on the
//      order of its increments.
#pragma once
#include <type_traits>

#include "gdbg_persist.cuh"

namespace gdbg {

constexpr int SP_EMIT_BLOCK = 256;
constexpr int SP_PART_BLOCK = 512;
constexpr int SP_APPLY_BLOCK = 512;
constexpr int SP_NBUF = 2;
constexpr uint64_t SP_EMPTY = ~0ull;

__device__ __forceinline__ uint64_t sp_records(const SortParams& sp) {
    const uint64_t nk = __ldg(sp.total_kmers);
    return (nk < sp.kmer_cap ? nk : sp.kmer_cap) * sp.n_tables;
}
__device__ __forceinline__ uint32_t sp_bucket(uint64_t rec, uint32_t fs) {
    return (uint32_t)(rec >> 32) >> fs;
}

// ---- bulk copies into shared memory ---------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a barrier phase; false when WAIT_CAP polls run out.  The
// last wait for copies still in flight before a block gives up always takes
// this limit, so no block leaves with a copy still writing its shared memory.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < WAIT_CAP; ++it)
        if (mbar_try(bar, parity)) return true;
    return false;
}
// Non-blocking test of a barrier phase.
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// First wait on a bulk copy: WAIT_CAP blocking polls, or, when the handle set
// a limit (SortParams::wait_cap), that many non-blocking tests, so a small
// limit runs out within nanoseconds of the copy's issue.
__device__ __forceinline__ bool copy_wait(const SortParams& sp, uint64_t* bar, uint32_t parity) {
    if (sp.wait_cap == 0) return mbar_wait(bar, parity);
    for (uint32_t it = 0; it < sp.wait_cap; ++it)
        if (mbar_test(bar, parity)) return true;
    return false;
}
// Global -> shared bulk copy; both addresses 16-byte aligned, bytes a
// multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// ---- 1. records and first-digit counts --------------------------------------

constexpr uint32_t SP_RUN = SP_SEGK / SP_EMIT_BLOCK;   // k-mers hashed by one thread

// Sequential 2-bit base reader.  A word is loaded only when a base of it is
// read (a cursor placed at the end of the stream reads nothing past it):
// `p` is the next word to load, `first` the base offset inside it, `left` the
// bases still in `word`.
struct EmitCursor {
    const uint32_t* __restrict__ p;
    uint32_t word, left, first;
    __device__ __forceinline__ void init(const uint32_t* packed, uint64_t pos) {
        p = packed + (pos >> 4);
        first = (uint32_t)(pos & 15u);
        left = 0;
    }
    __device__ __forceinline__ uint32_t next() {
        if (left == 0) {
            word = __ldg(p++) >> (first << 1);
            left = 16u - first;
            first = 0;
        }
        const uint32_t c = word & 3u;
        word >>= 2;
        --left;
        return c;
    }
};

// One block per segment of SP_SEGK k-mers; thread t hashes the run of SP_RUN
// consecutive k-mers starting at k-mer t * SP_RUN of the segment by rolling
// (re-seeding at read starts).  Record order inside a segment is free (the
// partition passes do not keep it), so step j of every thread goes to the
// segment slots j * (active threads) + t: each warp writes one contiguous
// run per step.
template <bool CANON, int NT, bool SMALLP>
__global__ void __launch_bounds__(SP_EMIT_BLOCK)
k_sp_emit(BatchView b, HashParams hp, TableParams tp, SortParams sp, uint64_t* __restrict__ rout,
          uint32_t seg0) {
    __shared__ __align__(16) uint64_t stage[NT == 4 ? 1 : SP_EMIT_BLOCK / 32][32 * BK_MAXNT];
    __shared__ uint32_t hist[256];
    // roll terms by (out, in): fw ^= symk(out) ^ sym(in), rc ^= symk(3-in) ^ sym(3-out)
    __shared__ uint64_t roll_fw[16], roll_rc[16];
    const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t s = seg0 + blockIdx.x;   // launches may cover a range of segments
    for (uint32_t k = tid; k < sp.bins1; k += SP_EMIT_BLOCK) hist[k] = 0;
    if (tid < 16) {
        const uint32_t out = tid >> 2, in = tid & 3u;
        roll_fw[tid] = symk(hp, out) ^ sym(in);
        roll_rc[tid] = symk(hp, 3u - in) ^ sym(3u - out);
    }
    __syncthreads();
    const uint64_t total = __ldg(b.kofs + b.n_reads);
    uint64_t nk = total < sp.kmer_cap ? total : sp.kmer_cap;
    if (nk > b.n_map_tiles * MAP_TILE) nk = b.n_map_tiles * MAP_TILE;
    const uint64_t gs = (uint64_t)s * SP_SEGK;
    const uint32_t m = gs < nk ? (uint32_t)(nk - gs < SP_SEGK ? nk - gs : SP_SEGK) : 0u;
    const uint32_t F = m / SP_RUN, P = m % SP_RUN;   // full runs, length of the partial one
    const uint32_t n = NT > 0 ? (uint32_t)NT : sp.n_tables;
    const uint32_t my_len = tid < F ? SP_RUN : (tid == F ? P : 0u);
    uint64_t r = 0, kend = 0, fw = 0, rc = 0;
    uint32_t left = 0;   // k-mers of the current read from the current one on
    EmitCursor cin, cout;
    const uint32_t K = hp.K;
    auto seed = [&](uint64_t g) {
        const uint64_t base = __ldg(b.offsets + r) + (g - __ldg(b.kofs + r));
        cin.init(b.packed, base);
        cout.init(b.packed, base);
        fw = 0;
        rc = 0;
        for (uint32_t i = 0; i < K; ++i) {
            const uint32_t c = cin.next();
            fw = rotl1(fw) ^ sym(c);
            if (CANON) rc ^= rotl64(sym(3u - c), i);
        }
    };
    if (my_len) {
        const uint64_t ga = gs + (uint64_t)tid * SP_RUN;
        r = find_read(b, ga, total);
        kend = __ldg(b.kofs + r + 1);
        left = (uint32_t)(kend - ga);
        seed(ga);
    }
    // ordinals are below 2^32; the records of step j start at slot slot0
    const uint32_t g0 = (uint32_t)gs + tid * SP_RUN;
    const uint32_t dsh = sp.fs + sp.hi_shift;   // first digit = cell >> dsh (dsh < 32)
    uint4* const obase = reinterpret_cast<uint4*>(rout + (gs + tid) * 4u);
    uint32_t slot0 = 0;
    const uint32_t n_steps = F ? SP_RUN : P;   // the longest run of the block
    for (uint32_t j = 0; j < n_steps; ++j) {
        const bool act = j < my_len;
        bool reseed = false;
        uint64_t rbase = 0;
        if (act && j > 0) {
            if (--left == 0) {
                const uint64_t g = gs + (uint64_t)tid * SP_RUN + j;
                do {
                    ++r;
                    kend = __ldg(b.kofs + r + 1);
                } while (kend <= g);
                left = (uint32_t)(kend - g);
                rbase = __ldg(b.offsets + r) + (g - __ldg(b.kofs + r));
                reseed = true;
            } else {
                const uint32_t out = cout.next();
                const uint32_t in = cin.next();
                // roll_right with the terms from the table
                fw = rotl1(fw) ^ roll_fw[out * 4u + in];
                if (CANON) rc = rotr1(rc ^ roll_rc[out * 4u + in]);
            }
        }
        // lanes that entered a new read: the warp computes each one's seed
        // together (one base per lane, XOR-reduced), instead of one lane
        // rolling K bases while the others wait
        uint32_t need = __ballot_sync(0xFFFFFFFFu, reseed);
        while (need) {
            const int L = __ffs(need) - 1;
            need &= need - 1;
            const uint64_t pb = __shfl_sync(0xFFFFFFFFu, rbase, L);
            uint64_t sf = 0, sr = 0;
            for (uint32_t i = lane; i < K; i += 32) {
                const uint32_t c = base_at(b.packed, pb + i);
                sf ^= rotl64(sym(c), (K - 1u - i) & 63u);
                if (CANON) sr ^= rotl64(sym(3u - c), i & 63u);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sf ^= __shfl_xor_sync(0xFFFFFFFFu, sf, o);
                if (CANON) sr ^= __shfl_xor_sync(0xFFFFFFFFu, sr, o);
            }
            if ((int)lane == L) {
                fw = sf;
                rc = sr;
                cin.init(b.packed, pb + K);
                cout.init(b.packed, pb);
            }
        }
        // slots of step j: threads active at step j, in thread order (the
        // active threads are 0 .. A-1, so thread t takes slot slot0 + t)
        const uint32_t A = j < P ? F + 1 : F;
        if (NT == 4) {
            if (act) {
                const uint64_t h = hash_value<CANON>(fw, rc);
                // global cells are below 2^32: 32-bit cell, bucket and digit
                uint32_t gc[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    gc[i] = (uint32_t)sp.tbase[i] + (SMALLP ? fastmod_small(h, (uint32_t)tp.p[i], tp.m[i])
                                                            : (uint32_t)fastmod(h, tp.p[i], tp.m[i]));
                    atomicAdd(&hist[gc[i] >> dsh], 1u);
                }
                // the slot's 4 records, (cell << 32) | ordinal, as two 16-byte
                // stores; consecutive threads write consecutive 32-byte slots
                const uint32_t gl = g0 + j;
                uint4* d4 = obase + 2u * slot0;
                d4[0] = make_uint4(gl, gc[0], gl, gc[1]);
                d4[1] = make_uint4(gl, gc[2], gl, gc[3]);
            }
        } else {
            if (act) {
                const uint64_t h = hash_value<CANON>(fw, rc);
#pragma unroll
                for (int i = 0; i < BK_MAXNT; ++i) {
                    if (i < (int)n) {
                        const uint32_t gc = (uint32_t)sp.tbase[i] +
                                            (SMALLP ? fastmod_small(h, (uint32_t)tp.p[i], tp.m[i])
                                                    : (uint32_t)fastmod(h, tp.p[i], tp.m[i]));
                        stage[w][lane * n + i] = ((uint64_t)gc << 32) | (g0 + j);
                        atomicAdd(&hist[gc >> dsh], 1u);
                    }
                }
            }
            __syncwarp();
            const uint32_t wa = A > w * 32 ? (A - w * 32 < 32 ? A - w * 32 : 32u) : 0u;
            if (wa) {
                uint64_t* dst = rout + (gs + slot0 + w * 32) * n;
                for (uint32_t k = lane; k < wa * n; k += 32) dst[k] = stage[w][k];
            }
            __syncwarp();
        }
        slot0 += A;
    }
    __syncthreads();
    for (uint32_t k = tid; k < sp.bins1; k += SP_EMIT_BLOCK)
        sp.hist1[(uint64_t)k * sp.nseg1 + s] = hist[k];
}

// ---- 3a. pass-2 segment plan -------------------------------------------------

// One block of 256 threads: group starts G[] from the pass-1 scan, segments
// per group, and their exclusive scan s0[].
__global__ void __launch_bounds__(256) k_sp_plan(SortParams sp) {
    __shared__ uint32_t ws[8];
    uint32_t* s0 = sp.plan;
    uint32_t* G = sp.plan + sp.bins1 + 1;
    const uint32_t g = threadIdx.x;
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    uint32_t start = 0, next = n_recs;
    if (g < sp.bins1) start = sp.off1[(uint64_t)g * sp.nseg1];
    if (g + 1 < sp.bins1) next = sp.off1[(uint64_t)(g + 1) * sp.nseg1];
    const uint32_t nseg = g < sp.bins1 ? (next - start + SP_SEG2 - 1) / SP_SEG2 : 0u;
    // block exclusive scan of nseg
    const uint32_t lane = g & 31, w = g >> 5;
    uint32_t inc = nseg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    uint32_t add = 0;
    for (uint32_t k = 0; k < w; ++k) add += ws[k];
    const uint32_t excl = add + inc - nseg;
    if (g < sp.bins1) {
        s0[g] = excl;
        G[g] = start;
    }
    if (g == sp.bins1 - 1) {
        s0[sp.bins1] = excl + nseg;
        G[sp.bins1] = n_recs;
    }
}

// Which group a pass-2 segment belongs to, and its record range.
struct Seg2 {
    uint32_t group, k, nseg, rs, re;
    bool valid;
};
__device__ __forceinline__ Seg2 seg2_of(const SortParams& sp, uint32_t s) {
    const uint32_t* s0 = sp.plan;
    const uint32_t* G = sp.plan + sp.bins1 + 1;
    Seg2 r{};
    r.valid = s < s0[sp.bins1] && s < sp.nseg2_cap;
    if (!r.valid) return r;
    uint32_t lo = 0, hi = sp.bins1;   // last group with s0[g] <= s
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s0[mid] <= s) lo = mid;
        else hi = mid;
    }
    r.group = lo;
    r.k = s - s0[lo];
    r.nseg = s0[lo + 1] - s0[lo];
    r.rs = G[lo] + r.k * SP_SEG2;
    const uint32_t e = r.rs + SP_SEG2;
    r.re = e < G[lo + 1] ? e : G[lo + 1];
    return r;
}

// ---- 3b. pass-2 counts ------------------------------------------------------

__global__ void __launch_bounds__(SP_PART_BLOCK)
k_sp_hist2(SortParams sp, const uint64_t* __restrict__ rin) {
    __shared__ uint32_t cnt[SP_MAXBINS2];
    __shared__ Seg2 sg;
    if (threadIdx.x == 0) sg = seg2_of(sp, blockIdx.x);
    for (uint32_t k = threadIdx.x; k < sp.bins2; k += SP_PART_BLOCK) cnt[k] = 0;
    __syncthreads();
    if (!sg.valid) return;
    const uint32_t mask = sp.bins2 - 1;
    constexpr int U = 8;   // loads in flight per thread
    for (uint32_t k0 = sg.rs + threadIdx.x; k0 < sg.re; k0 += U * SP_PART_BLOCK) {
        uint64_t v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t k = k0 + u * SP_PART_BLOCK;
            v[u] = k < sg.re ? __ldcs(rin + k) : SP_EMPTY;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (v[u] != SP_EMPTY) atomicAdd(&cnt[sp_bucket(v[u], sp.fs) & mask], 1u);
    }
    __syncthreads();
    const uint64_t base = (uint64_t)sp.bins2 * sp.plan[sg.group];
    for (uint32_t d = threadIdx.x; d < sp.bins2; d += SP_PART_BLOCK)
        sp.hist2[base + (uint64_t)d * sg.nseg + sg.k] = cnt[d];
}

// ---- 2 / 3c. partition passes -----------------------------------------------

constexpr uint32_t SP_BUF = SP_TILE + 2;   // records per input buffer (alignment slack)

__host__ __device__ constexpr size_t sp_part_smem() {
    return (size_t)(SP_NBUF * SP_BUF + SP_TILE) * 8;
}

template <bool PASS2>
__global__ void __launch_bounds__(SP_PART_BLOCK, 2)
k_sp_part(SortParams sp, const uint64_t* __restrict__ rin, uint64_t* __restrict__ rout) {
    extern __shared__ __align__(128) uint64_t sm[];
    uint64_t* inbuf = sm;                       // SP_NBUF x SP_BUF
    uint64_t* stage = sm + SP_NBUF * SP_BUF;    // SP_TILE
    constexpr uint32_t MB = PASS2 ? SP_MAXBINS2 : 256u;
    __shared__ uint32_t cnt[MB], lstart[MB], cursor[MB], delta[MB];
    __shared__ uint32_t wsum[SP_PART_BLOCK / 32];
    __shared__ __align__(8) uint64_t bars[SP_NBUF];
    __shared__ uint32_t rs_s, re_s, abort_s;
    const uint32_t tid = threadIdx.x;
    const uint32_t bins = PASS2 ? sp.bins2 : sp.bins1;
    if (tid == 0) {
        uint32_t rs = 0, re = 0;
        if (PASS2) {
            const Seg2 sg = seg2_of(sp, blockIdx.x);
            if (sg.valid) {
                rs = sg.rs;
                re = sg.re;
            }
        } else {
            const uint64_t nr = sp_records(sp);
            const uint64_t a = (uint64_t)blockIdx.x * SP_SEGK * sp.n_tables;
            const uint64_t e = a + (uint64_t)SP_SEGK * sp.n_tables;
            rs = (uint32_t)(a < nr ? a : nr);
            re = (uint32_t)(e < nr ? e : nr);
        }
        rs_s = rs;
        re_s = re;
        abort_s = 0;
        for (int i = 0; i < SP_NBUF; ++i) mbar_init(&bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint32_t rs = rs_s, re = re_s;
    if (rs >= re) return;
    // segment cursors
    if (PASS2) {
        const Seg2 sg = seg2_of(sp, blockIdx.x);
        const uint64_t base = (uint64_t)sp.bins2 * sp.plan[sg.group];
        for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK)
            cursor[d] = sp.off2[base + (uint64_t)d * sg.nseg + sg.k];
    } else {
        for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK)
            cursor[d] = sp.off1[(uint64_t)d * sp.nseg1 + blockIdx.x];
    }
    const uint32_t n_tiles = (re - rs + SP_TILE - 1) / SP_TILE;
    // digit of a record: (cell >> (fs + shift)) & mask
    const uint32_t dshift = sp.fs + (PASS2 ? 0u : sp.hi_shift);
    const uint32_t mask = PASS2 ? sp.bins2 - 1 : 0xFFFFFFFFu;
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    const uint32_t lane = tid & 31u, w = tid >> 5;
    // tile i covers records [rs + i*SP_TILE, ...); its copy starts at the
    // even index at or below, so the copy is 16-byte aligned and sized
    auto issue = [&](uint32_t i) {
        const uint32_t ts = rs + i * SP_TILE;
        const uint32_t te = ts + SP_TILE < re ? ts + SP_TILE : re;
        const uint32_t a0 = ts & ~1u, a1 = (te + 1) & ~1u;
        uint64_t* bar = &bars[i % SP_NBUF];
        mbar_expect(bar, (a1 - a0) * 8u);
        bulk_load(inbuf + (i % SP_NBUF) * SP_BUF, rin + a0, (a1 - a0) * 8u, bar);
    };
    for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK) cnt[d] = 0;
    if (tid == 0)
        for (uint32_t i = 0; i < SP_NBUF && i < n_tiles; ++i) issue(i);
    constexpr int IPT = SP_TILE / SP_PART_BLOCK;
    for (uint32_t i = 0; i < n_tiles; ++i) {
        const uint32_t ts = rs + i * SP_TILE;
        const uint32_t nt = re - ts < SP_TILE ? re - ts : SP_TILE;
        const uint64_t* src = inbuf + (i % SP_NBUF) * SP_BUF + (ts & 1u);
        if (!copy_wait(sp, &bars[i % SP_NBUF], (i / SP_NBUF) & 1u)) atomicExch(&abort_s, 1u);
        // also orders the previous tile's reads of stage / delta before this
        // tile's writes
        __syncthreads();
        if (abort_s) {
            // give the copies in flight a last bounded wait, then leave
            if (tid == 0) {
                atomicOr(sp.err, GDBG_ERR_COPY_TIMEOUT);
                for (uint32_t j = i; j < i + SP_NBUF && j < n_tiles; ++j)
                    mbar_wait(&bars[j % SP_NBUF], (j / SP_NBUF) & 1u);
            }
            return;
        }
        // ranks inside the tile: all loads first, then all atomics
        uint64_t r[IPT];
        uint32_t dg[IPT], pos[IPT];
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const uint32_t k = j * SP_PART_BLOCK + tid;
            r[j] = k < nt ? src[k] : 0;
        }
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const uint32_t k = j * SP_PART_BLOCK + tid;
            dg[j] = ((uint32_t)(r[j] >> 32) >> dshift) & mask;
            pos[j] = k < nt ? atomicAdd(&cnt[dg[j]], 1u) : 0u;
        }
        __syncthreads();
        // buffer consumed: refill it with tile i + SP_NBUF
        if (tid == 0 && i + SP_NBUF < n_tiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(i + SP_NBUF);
        }
        // tile-local bin starts: one bin per thread, warp scans, then the
        // warps' totals; delta[d] = global base - local start
        const uint32_t c = tid < bins ? cnt[tid] : 0u;
        if (tid < bins) cnt[tid] = 0;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= (uint32_t)o) inc += y;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (tid < bins) {
            uint32_t pre = 0;
            for (uint32_t q = 0; q < w; ++q) pre += wsum[q];
            const uint32_t ex = pre + inc - c;
            lstart[tid] = ex;
            delta[tid] = cursor[tid] - ex;
            cursor[tid] += c;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const uint32_t k = j * SP_PART_BLOCK + tid;
            if (k < nt) stage[lstart[dg[j]] + pos[j]] = r[j];
        }
        __syncthreads();
        // runs of equal digits go out contiguously
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const uint32_t k = j * SP_PART_BLOCK + tid;
            if (k < nt) {
                const uint64_t v = stage[k];
                const uint32_t p = delta[((uint32_t)(v >> 32) >> dshift) & mask] + k;
                if (p < n_recs) rout[p] = v;
                else atomicOr(sp.err, GDBG_ERR_PARTITION);
            }
        }
    }
}

// ---- 3d. bucket starts ---------------------------------------------------------

__global__ void k_sp_starts(SortParams sp, uint32_t* __restrict__ start) {
    const uint32_t bk = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    if (bk > sp.n_buckets) return;
    if (bk == sp.n_buckets) {
        start[bk] = n_recs;
        return;
    }
    if (sp.bins2 == 1) {
        start[bk] = sp.off1[(uint64_t)bk * sp.nseg1];
        return;
    }
    const uint32_t* s0 = sp.plan;
    const uint32_t* G = sp.plan + sp.bins1 + 1;
    const uint32_t g = bk >> sp.hi_shift, d = bk & (sp.bins2 - 1);
    const uint32_t nseg = s0[g + 1] - s0[g];
    start[bk] = nseg ? sp.off2[(uint64_t)sp.bins2 * s0[g] + (uint64_t)d * nseg] : G[g];
}

// ---- 4. order-independent apply -------------------------------------------

// Shared memory of the apply: a bucket's records staged at once (up to
// SortParams::rbuf_cap of them), its table region, and one map space used
// two ways.  The single-chunk path (all of a bucket's records staged) keys
// each zero cell to the staged record with the smallest ordinal, in 32-bit
// entries (cell << idx_bits | record index); the chunked path (buckets of
// more records than the buffer holds) keeps 64-bit entries (ordinal << 32 |
// cell) and restages records per cell range.  The kernel is issue-bound, so
// the launcher sizes the record buffer for the batch's expected bucket load
// and the map space (8 or 16 KB) for the most CTAs per SM that leaves: three
// with 32 KB regions, four with small regions and light buckets.
constexpr uint32_t SP_RBUF_MIN = 4096, SP_RBUF_MAX = 8192;   // records staged at once
constexpr uint32_t SP_MAP_MIN = 8192, SP_MAP_MAX = 16384;    // map space bytes
constexpr uint32_t SP_EMPTY32 = 0xFFFFFFFFu;
// Linear-probe limit of a map insert.  A map filled to half its slots needs
// about two probes; a fuller one -- a fresh, empty table puts nearly every
// cell of a region into the map -- would make each insert walk the whole map,
// so an insert that runs this long reports the map full and the cell range is
// narrowed.
constexpr uint32_t SP_PROBE_CAP = 64;

__device__ __forceinline__ uint32_t sp_slot_bits(uint32_t co, uint32_t bits) {
    return (co * 0x9E3779B1u) >> (32 - bits);
}

// Shared-memory layout of k_sp_apply (byte offsets): region words (padded
// to 16 bytes), map space, record buffer (+2 alignment slack), dirty
// sector bits.
struct ApplyLayout {
    uint32_t map_off, rec_off, dirty_off, total;
};
__host__ __device__ constexpr ApplyLayout sp_apply_layout(uint32_t region_words, uint32_t map_b,
                                                         uint32_t rbuf_cap) {
    const uint32_t region_b = ((region_words + 3u) & ~3u) * 4u;
    const uint32_t rec_b = (rbuf_cap + 2u) * 8u;
    const uint32_t dirty_b = (((region_words + 7u) / 8u + 31u) / 32u) * 4u;
    return ApplyLayout{region_b, region_b + map_b, region_b + map_b + rec_b,
                       region_b + map_b + rec_b + dirty_b};
}

// After pass 1 the map holds every cell of the range that was zero before
// the batch, with the minimum ordinal of its records: that k-mer is the
// cell's first toucher, so it is new.  Each thread reads its own slots.
__device__ __forceinline__ void sp_map_winners(const uint64_t* map, uint32_t slots,
                                               const SortParams& sp, int ti,
                                               uint32_t* __restrict__ new_bits,
                                               unsigned long long& occ) {
    for (uint32_t k = threadIdx.x; k < slots; k += SP_APPLY_BLOCK) {
        const uint64_t e = map[k];
        if (e == SP_EMPTY) continue;
        const uint32_t g = (uint32_t)(e >> 32);
        if (g < sp.kmer_cap) {
            atomicOr(new_bits + (g >> 5), 1u << (g & 31u));
            if (ti == 0) ++occ;
        }
    }
}

// Chunked-path map insert of a zero cell with ordinal g (2^bits slots): the
// slot index, or the slot count when the map is full; *created is set when
// this call made the entry.
__device__ __forceinline__ uint32_t sp_map_insert(uint64_t* map, uint32_t bits, uint32_t co,
                                                  uint32_t g, bool* created) {
    const uint32_t slots = 1u << bits;
    const uint64_t mine = ((uint64_t)g << 32) | co;   // (ordinal << 32) | cell
    uint32_t sl = sp_slot_bits(co, bits);
    *created = false;
    for (uint32_t it = 0; it < SP_PROBE_CAP; ++it) {
        uint64_t cur = map[sl];
        if (cur == SP_EMPTY) {
            cur = atomicCAS((unsigned long long*)&map[sl], SP_EMPTY, mine);
            if (cur == SP_EMPTY) {
                *created = true;
                return sl;
            }
        }
        if ((uint32_t)cur == co) {
            if (mine < cur) atomicMin((unsigned long long*)&map[sl], mine);
            return sl;
        }
        sl = (sl + 1) & (slots - 1);
    }
    return slots;
}

// Single-chunk map insert (2^bits slots): zero cell co touched by staged
// record k (below 2^ib).  The slot keeps the cell's record with the
// smallest ordinal (records of one bucket never share an ordinal: a k-mer
// has one cell per table).  Returns the slot, or the slot count when the map
// is full; *created when this call made it.
__device__ __forceinline__ uint32_t sp_map32_insert(uint32_t* map, uint32_t bits, uint32_t ib,
                                                    const uint64_t* src, uint32_t co, uint32_t k,
                                                    bool* created) {
    const uint32_t slots = 1u << bits, im = (1u << ib) - 1u;
    const uint32_t mine = (co << ib) | k;
    const uint32_t g = (uint32_t)src[k];
    uint32_t sl = sp_slot_bits(co, bits);
    *created = false;
    for (uint32_t it = 0; it < SP_PROBE_CAP; ++it) {
        uint32_t cur = map[sl];
        if (cur == SP_EMPTY32) {
            cur = atomicCAS(map + sl, SP_EMPTY32, mine);
            if (cur == SP_EMPTY32) {
                *created = true;
                return sl;
            }
        }
        if ((cur >> ib) == co) {
            // the same cell: this record takes the slot while its ordinal is
            // smaller (each successful swap lowers the ordinal held)
            for (uint32_t t = 0; t < slots && (uint32_t)src[cur & im] > g; ++t) {
                const uint32_t prev = atomicCAS(map + sl, cur, mine);
                if (prev == cur) break;
                cur = prev;
            }
            return sl;
        }
        sl = (sl + 1) & (slots - 1);
    }
    return slots;
}

// Saturating increment of one region cell; true when the word changed.
template <int STORAGE>
__device__ __forceinline__ bool sp_increment(uint32_t* region, uint32_t word, uint32_t shift) {
    if (STORAGE == GDBG_BIT) {
        const uint32_t bit = 1u << shift;
        return (atomicOr(region + word, bit) & bit) == 0;
    }
    uint32_t cur = region[word];
    for (int it = 0; it < (1 << 20); ++it) {
        if (cell_value<STORAGE>(cur, shift) >= cell_max<STORAGE>()) return false;
        const uint32_t prev = atomicCAS(region + word, cur, cur + (1u << shift));
        if (prev == cur) return true;
        cur = prev;
    }
    return false;
}

// One CTA per bucket; the region and the bucket's records are bulk-copied
// into shared memory.  Pass 1 puts every cell that is zero in the region
// into the map with the minimum k-mer ordinal of its records; pass 2 applies
// every record (saturating increment) and flags the map's minimum as new.
// A bucket whose records fit one staging buffer keeps each record's map slot
// from pass 1 (pass 2 looks up nothing); larger or denser buckets take the
// general loop over buffer chunks and cell ranges.
// MAPB: map space bytes (SortParams::map_bytes), IB: record-index bits of a
// single-chunk map entry (SortParams::idx_bits); compile-time, so the map's
// hashing and entry packing take no run-time shifts.
template <int STORAGE, uint32_t MAPB, uint32_t IB>
__global__ void __launch_bounds__(SP_APPLY_BLOCK, 4)
k_sp_apply(TableParams tp, SortParams sp, const uint64_t* __restrict__ recs,
           const uint32_t* __restrict__ start, uint32_t* __restrict__ new_bits,
           unsigned long long* counters) {
    extern __shared__ __align__(128) unsigned char sbytes[];
    __shared__ uint32_t n_fresh, overflow, abort_s;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t used[SP_MAP_MAX / 4 / 32];   // single-chunk map slots created
    const uint32_t bk = blockIdx.x;
    const uint32_t rs = start[bk], re = start[bk + 1];
    if (rs >= re) return;
    int ti = 0;
    while (ti + 1 < tp.n && sp.bbase[ti + 1] <= bk) ++ti;
    const uint32_t region_cells = 1u << sp.fs;
    const uint32_t region_words = region_cells / cells_per_word<STORAGE>();
    const uint32_t region_sectors = (region_words + 7) / 8;
    const uint32_t RB = sp.rbuf_cap;   // records staged at once
    const ApplyLayout L = sp_apply_layout(region_words, sp.map_bytes, RB);
    // map slots: 32-bit entries for the single-chunk path, 64-bit for the chunked one
    constexpr uint32_t slots32 = MAPB / 4u, bits32 = slots32 == 4096u ? 12u : 11u;
    // entries (cell << IB | index) never reach the all-ones empty entry
    if (sp.fs + IB > 31u) {
        if (threadIdx.x == 0) atomicOr(sp.err, GDBG_ERR_PARTITION);
        return;
    }
    constexpr uint32_t bits64 = bits32 - 1u, slots64 = 1u << bits64;
    static_assert((1u << bits32) == slots32, "map space of 8 or 16 KB");
    uint32_t* region = reinterpret_cast<uint32_t*>(sbytes);
    uint64_t* map = reinterpret_cast<uint64_t*>(sbytes + L.map_off);     // chunked path
    uint32_t* map32 = reinterpret_cast<uint32_t*>(sbytes + L.map_off);   // single-chunk path
    uint64_t* rbuf = reinterpret_cast<uint64_t*>(sbytes + L.rec_off);
    uint32_t* dirty = reinterpret_cast<uint32_t*>(sbytes + L.dirty_off);
    const uint64_t c0 = (uint64_t)(bk - sp.bbase[ti]) << sp.fs;
    const uint64_t w0 = c0 / cells_per_word<STORAGE>();
    uint32_t nw = region_words;
    if (w0 + nw > sp.twords[ti]) nw = (uint32_t)(sp.twords[ti] - w0);
    const uint32_t* gsrc = tp.words[ti] + w0;
    // the region by one bulk copy when it is a whole number of 16-byte units
    const bool bulk_region = ((w0 & 3u) == 0) && ((nw & 3u) == 0);
    const uint32_t n_recs = re - rs;
    const uint32_t n_chunks = (n_recs + RB - 1) / RB;
    // dense buckets write the whole region back; sparse ones their dirty sectors
    const bool track = n_recs < region_sectors;
    uint32_t phase = 0;
    // records of chunk c into rbuf, copied from the even index at or below
    // its first record (and the region with chunk 0)
    auto chunk_copy = [&](uint32_t c, bool with_region) {
        const uint32_t a = rs + c * RB;
        const uint32_t b = a + RB < re ? a + RB : re;
        const uint32_t a0 = a & ~1u, a1 = (b + 1) & ~1u;
        const uint32_t bytes = (a1 - a0) * 8u + (with_region ? nw * 4u : 0u);
        mbar_expect(&bar, bytes);
        if (with_region) bulk_load(region, gsrc, nw * 4u, &bar);
        bulk_load(rbuf, recs + a0, (a1 - a0) * 8u, &bar);
    };
    if (threadIdx.x == 0) {
        abort_s = 0;
        n_fresh = 0;
        overflow = 0;
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        chunk_copy(0, bulk_region);
    }
    if (!bulk_region)
        for (uint32_t k = threadIdx.x; k < nw; k += SP_APPLY_BLOCK) region[k] = __ldcs(gsrc + k);
    if (track)
        for (uint32_t k = threadIdx.x; k < (region_sectors + 31) / 32; k += SP_APPLY_BLOCK) dirty[k] = 0;
    for (uint32_t k = threadIdx.x; k < slots32; k += SP_APPLY_BLOCK) map32[k] = SP_EMPTY32;
    for (uint32_t k = threadIdx.x; k < slots32 / 32; k += SP_APPLY_BLOCK) used[k] = 0;
    __syncthreads();   // the barrier is initialised before anyone waits on it
    if (!copy_wait(sp, &bar, phase & 1u)) atomicExch(&abort_s, 1u);
    ++phase;
    __syncthreads();
    if (abort_s) {
        if (threadIdx.x == 0) {
            atomicOr(sp.err, GDBG_ERR_COPY_TIMEOUT);
            mbar_wait(&bar, (phase - 1) & 1u);
        }
        return;
    }
    const uint32_t co_mask = region_cells - 1;
    unsigned long long occ = 0;
    bool done = false;
    if (n_chunks == 1) {
        // all records staged: the whole region as one cell range first, then,
        // when its zero cells overflow the map, narrower ranges
        const uint64_t* src = rbuf + (rs & 1u);
        constexpr uint32_t ib = IB, im = (1u << IB) - 1u;
        // pass 1 over [lo, hi): the staged record with the minimum ordinal per
        // zero cell; true when the range fits the map
        // (generic lambdas: the whole-region form is compiled without the
        // range test)
        auto map_pass = [&](auto whole_c, uint32_t lo, uint32_t hi) -> bool {
            constexpr bool whole = decltype(whole_c)::value;
            uint32_t inserted = 0;
            bool lost = false;
            for (uint32_t k = threadIdx.x; k < n_recs; k += SP_APPLY_BLOCK) {
                const uint64_t rec = src[k];
                const uint32_t co = (uint32_t)(rec >> 32) & co_mask;
                if (!whole && (co < lo || co >= hi)) continue;
                uint32_t word, shift;
                region_cell<STORAGE>(co, word, shift);
                // once the map has overflowed the range is redone narrower:
                // the remaining inserts are skipped
                if (cell_value<STORAGE>(region[word], shift) == 0 && !*(volatile uint32_t*)&overflow) {
                    bool created;
                    const uint32_t sl = sp_map32_insert(map32, bits32, ib, src, co, k, &created);
                    inserted += created;
                    if (sl >= slots32) {
                        lost = true;
                        overflow = 1;
                    }
                    if (created) atomicOr(&used[sl >> 5], 1u << (sl & 31u));
                }
            }
            inserted = __reduce_add_sync(0xFFFFFFFFu, inserted);
            if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(&n_fresh, inserted);
            if (lost) overflow = 1;
            __syncthreads();
            return !overflow && n_fresh <= slots32 / 2;
        };
        // pass 2 over [lo, hi): every record applied; then the map's entries
        // (the first touchers) flagged new
        auto apply_pass = [&](auto whole_c, uint32_t lo, uint32_t hi) {
            constexpr bool whole = decltype(whole_c)::value;
            for (uint32_t k = threadIdx.x; k < n_recs; k += SP_APPLY_BLOCK) {
                const uint64_t rec = src[k];
                const uint32_t co = (uint32_t)(rec >> 32) & co_mask;
                if (!whole && (co < lo || co >= hi)) continue;
                uint32_t word, shift;
                region_cell<STORAGE>(co, word, shift);
                const bool changed = sp_increment<STORAGE>(region, word, shift);
                if (track && changed) {
                    const uint32_t sec = word >> 3;
                    atomicOr(dirty + (sec >> 5), 1u << (sec & 31u));
                }
            }
            for (uint32_t wd = threadIdx.x; wd < slots32 / 32; wd += SP_APPLY_BLOCK) {
                for (uint32_t m = used[wd]; m; m &= m - 1) {
                    const uint32_t g = (uint32_t)src[map32[wd * 32 + __ffs(m) - 1] & im];
                    if (g < sp.kmer_cap) {
                        atomicOr(new_bits + (g >> 5), 1u << (g & 31u));
                        if (ti == 0) ++occ;
                    }
                }
            }
        };
        auto clear_map = [&]() {
            __syncthreads();   // everyone is done with the map and the counts
            for (uint32_t k = threadIdx.x; k < slots32; k += SP_APPLY_BLOCK) map32[k] = SP_EMPTY32;
            for (uint32_t k = threadIdx.x; k < slots32 / 32; k += SP_APPLY_BLOCK) used[k] = 0;
            if (threadIdx.x == 0) {
                n_fresh = 0;
                overflow = 0;
            }
            __syncthreads();
        };
        using whole_t = std::true_type;
        using ranged_t = std::false_type;
        if (map_pass(whole_t{}, 0, region_cells)) {
            apply_pass(whole_t{}, 0, region_cells);
        } else {
            uint32_t lo = 0, width = region_cells >> 1;
            for (int guard = 0; lo < region_cells && guard < 4096; ++guard) {
                const uint32_t hi = lo + width < region_cells ? lo + width : region_cells;
                clear_map();
                if (!map_pass(ranged_t{}, lo, hi) && width > 1) {
                    width >>= 1;   // redo this range narrower; nothing was applied yet
                    continue;
                }
                apply_pass(ranged_t{}, lo, hi);
                lo = hi;
            }
            if (lo < region_cells && threadIdx.x == 0) atomicOr(sp.err, GDBG_ERR_CLAIMS_FULL);
        }
        __syncthreads();
        done = true;
    }
    if (!done) {
        uint32_t loaded = 0;   // chunk in rbuf
        // all threads: make chunk c the one in rbuf (no-op when it already is)
        auto need_chunk = [&](uint32_t c) -> bool {
            if (c == loaded) return true;
            __syncthreads();   // everyone is done with the old chunk
            if (threadIdx.x == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                chunk_copy(c, false);
            }
            if (!copy_wait(sp, &bar, phase & 1u)) atomicExch(&abort_s, 1u);
            ++phase;
            __syncthreads();
            loaded = c;
            return abort_s == 0;
        };
        // cell ranges [lo, lo + width): narrower when the zero cells of a
        // range overflow the map
        uint32_t lo = 0, width = region_cells;
        int guard = 0;
        bool ok = true;
        for (; ok && lo < region_cells && guard < 4096; ++guard) {
            const uint32_t hi = lo + width < region_cells ? lo + width : region_cells;
            for (uint32_t k = threadIdx.x; k < slots64; k += SP_APPLY_BLOCK) map[k] = SP_EMPTY;
            if (threadIdx.x == 0) {
                n_fresh = 0;
                overflow = 0;
            }
            __syncthreads();
            // pass 1: minimum ordinal per zero cell
            uint32_t inserted = 0;
            bool lost = false;
            for (uint32_t c = 0; c < n_chunks && ok; ++c) {
                ok = need_chunk(c);
                if (!ok) break;
                const uint32_t a = rs + c * RB;
                const uint32_t cnt = re - a < RB ? re - a : RB;
                const uint64_t* src = rbuf + (a & 1u);
                for (uint32_t k = threadIdx.x; k < cnt; k += SP_APPLY_BLOCK) {
                    const uint64_t rec = src[k];
                    const uint32_t co = (uint32_t)(rec >> 32) & co_mask;
                    if (co < lo || co >= hi) continue;
                    uint32_t word, shift;
                    region_cell<STORAGE>(co, word, shift);
                    if (cell_value<STORAGE>(region[word], shift) != 0) continue;
                    if (*(volatile uint32_t*)&overflow) continue;   // redone narrower anyway
                    bool created;
                    const uint32_t sl = sp_map_insert(map, bits64, co, (uint32_t)rec, &created);
                    inserted += created;
                    if (sl >= slots64) {
                        lost = true;
                        overflow = 1;
                    }
                }
            }
            if (!ok) break;
            inserted = __reduce_add_sync(0xFFFFFFFFu, inserted);
            if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(&n_fresh, inserted);
            if (lost) overflow = 1;
            __syncthreads();
            if ((overflow || n_fresh > slots64 / 2) && width > 1) {
                width >>= 1;   // redo this range narrower; nothing was applied yet
                __syncthreads();
                continue;
            }
            // pass 2: apply every record of the range; the map's minima are new
            for (uint32_t c = 0; c < n_chunks && ok; ++c) {
                ok = need_chunk(c);
                if (!ok) break;
                const uint32_t a = rs + c * RB;
                const uint32_t cnt = re - a < RB ? re - a : RB;
                const uint64_t* src = rbuf + (a & 1u);
                for (uint32_t k = threadIdx.x; k < cnt; k += SP_APPLY_BLOCK) {
                    const uint64_t rec = src[k];
                    const uint32_t co = (uint32_t)(rec >> 32) & co_mask;
                    if (co < lo || co >= hi) continue;
                    uint32_t word, shift;
                    region_cell<STORAGE>(co, word, shift);
                    const bool changed = sp_increment<STORAGE>(region, word, shift);
                    if (track && changed) {
                        const uint32_t sec = word >> 3;
                        atomicOr(dirty + (sec >> 5), 1u << (sec & 31u));
                    }
                }
            }
            if (!ok) break;
            sp_map_winners(map, slots64, sp, ti, new_bits, occ);
            __syncthreads();
            lo = hi;
        }
        if (!ok) {
            // a copy wait ran out: flag it, give that copy one more bounded wait, leave
            if (threadIdx.x == 0) {
                atomicOr(sp.err, GDBG_ERR_COPY_TIMEOUT);
                mbar_wait(&bar, (phase - 1) & 1u);
            }
            return;
        }
        if (lo < region_cells && threadIdx.x == 0) atomicOr(sp.err, GDBG_ERR_CLAIMS_FULL);
    }
    // write back the region: every sector of a dense bucket, the dirty ones
    // of a sparse one (8 words each)
    uint32_t* gdst = tp.words[ti] + w0;
    for (uint32_t sec = threadIdx.x; sec < region_sectors; sec += SP_APPLY_BLOCK) {
        if (track && !((dirty[sec >> 5] >> (sec & 31u)) & 1u)) continue;
        const uint32_t wb = sec * 8;
        if (bulk_region && wb + 8 <= nw) {
            uint4* g4 = reinterpret_cast<uint4*>(gdst + wb);
            const uint4* s4 = reinterpret_cast<const uint4*>(region + wb);
            g4[0] = s4[0];
            g4[1] = s4[1];
        } else {
            for (uint32_t k = wb; k < wb + 8 && k < nw; ++k) gdst[k] = region[k];
        }
    }
    occ = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)occ);
    if ((threadIdx.x & 31) == 0 && occ) atomicAdd(counters + 1, occ);
}

__host__ __device__ constexpr size_t sp_apply_smem(uint32_t region_words, uint32_t map_b,
                                                   uint32_t rbuf_cap) {
    return sp_apply_layout(region_words, map_b, rbuf_cap).total;
}

}  // namespace gdbg
