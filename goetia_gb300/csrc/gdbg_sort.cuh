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
//      With four tables, k_sp_emit_part (gdbg_emit_part.cuh) does 1 and 2
//      in one kernel into a reserved layout, and these two run (gated) only
//      when one of its groups outgrew its slots.
//   3. k_sp_plan / k_sp_part<true, true>: every digit group is cut into
//      segments of SP_SEG2 records that never cross a group and partitioned
//      again by the low digit, each bucket's runs into its reserved slots.
//      k_sp_hist2 / its scan / k_sp_part<true, false> make the counted layout
//      instead (scan entries laid out group by group, so they are final
//      record positions), gated on a bucket outgrowing its slots.
//   4. k_sp_apply: one CTA per bucket bulk-copies its table region into
//      shared memory and reads the bucket's records, which are in no
//      particular order, once.  A cell that was not zero before the batch
//      takes its saturating increments at once; a zero cell stays zero
//      while a shared-memory map counts its touches and keeps the minimum
//      k-mer ordinal among them -- its first toucher, which is new -- and
//      gets min(max, touches) after the last record.  Zero cells that
//      overflow the map are redone in narrower cell ranges.  That is the
//      reference's sequential rule (bitstorage.hh:195-219, bytestorage.cc:
//      60-113, nibblestorage.cc:60-100) cell by cell; a cell's final value
//      does not depend on the order of its increments.
#pragma once

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
    // behind the fused emit: only when a group outgrew its reserved slots
    if (sp.gate1 && *(volatile const uint32_t*)sp.gate1 == 0) return;
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

// One block of 256 threads.  plan = s0[bins1 + 1] (exclusive scan of the
// segments per group), G[bins1 + 1] (each group's first record), GE[bins1 +
// 1] (its end) and D[bins1 + 1] (the records of the groups before it: where
// the group starts in the counted pass-2 layout).  The groups are the
// pass-1 output: dense (counted, from the emit's counts) or each in its
// reserved slot range (the fused emit) -- whichever pass 1 made.
__global__ void __launch_bounds__(256) k_sp_plan(SortParams sp) {
    __shared__ uint32_t ws[8], wd[8];
    uint32_t* s0 = sp.plan;
    uint32_t* G = sp.plan + (sp.bins1 + 1);
    uint32_t* GE = sp.plan + 2 * (sp.bins1 + 1);
    uint32_t* D = sp.plan + 3 * (sp.bins1 + 1);
    const uint32_t g = threadIdx.x;
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    const bool reserved1 = sp.gcap != nullptr && *(volatile const uint32_t*)sp.spill1 == 0;
    uint32_t start = 0, next = 0;
    if (g < sp.bins1) {
        if (reserved1) {
            start = sp.gbase[g];
            next = start + sp.gfill[g];
        } else {
            start = sp.off1[(uint64_t)g * sp.nseg1];
            next = g + 1 < sp.bins1 ? sp.off1[(uint64_t)(g + 1) * sp.nseg1] : n_recs;
        }
    }
    const uint32_t size = next - start;
    const uint32_t nseg = g < sp.bins1 ? (size + SP_SEG2 - 1) / SP_SEG2 : 0u;
    // block exclusive scans of nseg and size
    const uint32_t lane = g & 31, w = g >> 5;
    uint32_t inc = nseg, incd = size;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        const uint32_t yd = __shfl_up_sync(0xFFFFFFFFu, incd, o);
        if (lane >= o) {
            inc += y;
            incd += yd;
        }
    }
    if (lane == 31) {
        ws[w] = inc;
        wd[w] = incd;
    }
    __syncthreads();
    uint32_t add = 0, addd = 0;
    for (uint32_t k = 0; k < w; ++k) {
        add += ws[k];
        addd += wd[k];
    }
    const uint32_t excl = add + inc - nseg, excld = addd + incd - size;
    if (g < sp.bins1) {
        s0[g] = excl;
        G[g] = start;
        GE[g] = next;
        D[g] = excld;
    }
    if (g == sp.bins1 - 1) {
        s0[sp.bins1] = excl + nseg;
        G[sp.bins1] = next;
        GE[sp.bins1] = next;
        D[sp.bins1] = excld + size;
    }
}

// Which group a pass-2 segment belongs to, and its record range.
struct Seg2 {
    uint32_t group, k, nseg, rs, re;
    bool valid;
};
__device__ __forceinline__ Seg2 seg2_of(const SortParams& sp, uint32_t s) {
    const uint32_t* s0 = sp.plan;
    const uint32_t* G = sp.plan + (sp.bins1 + 1);
    const uint32_t* GE = sp.plan + 2 * (sp.bins1 + 1);
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
    r.re = e < GE[lo] ? e : GE[lo];
    return r;
}

// ---- 3b. pass-2 counts ------------------------------------------------------

__global__ void __launch_bounds__(SP_PART_BLOCK)
k_sp_hist2(SortParams sp, const uint64_t* __restrict__ rin) {
    __shared__ uint32_t cnt[SP_MAXBINS2];
    __shared__ Seg2 sg;
    // only for the counted layout: not needed when the reserved one held
    if (sp.bcap[0] != 0 && *(volatile const uint32_t*)sp.spill == 0) return;
    const uint32_t mask = sp.bins2 - 1;
    for (uint32_t s = blockIdx.x; s < sp.nseg2_cap; s += gridDim.x) {
        __syncthreads();   // the previous segment's counts are written out
        if (threadIdx.x == 0) sg = seg2_of(sp, s);
        for (uint32_t k = threadIdx.x; k < sp.bins2; k += SP_PART_BLOCK) cnt[k] = 0;
        __syncthreads();
        if (!sg.valid) {
            // past the last segment: the scan's tail entries, zeroed here
            const uint64_t tail = (uint64_t)sp.bins2 * s;
            for (uint32_t d = threadIdx.x; d < sp.bins2; d += SP_PART_BLOCK) sp.hist2[tail + d] = 0;
            continue;
        }
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
}

// ---- 2 / 3c. partition passes -----------------------------------------------

constexpr uint32_t SP_BUF = SP_TILE + 2;   // records per input buffer (alignment slack)

__host__ __device__ constexpr size_t sp_part_smem() {
    return (size_t)(SP_NBUF * SP_BUF + SP_TILE) * 8;
}

// PASS2 && RESERVE: the reserved layout (places taken per tile by atomics);
// PASS2 && !RESERVE: the counted layout, which does nothing when the
// reserved one was made and held.
template <bool PASS2, bool RESERVE>
__global__ void __launch_bounds__(SP_PART_BLOCK, 2)
k_sp_part(SortParams sp, const uint64_t* __restrict__ rin, uint64_t* __restrict__ rout) {
    extern __shared__ __align__(128) uint64_t sm[];
    uint64_t* inbuf = sm;                       // SP_NBUF x SP_BUF
    uint64_t* stage = sm + SP_NBUF * SP_BUF;    // SP_TILE
    constexpr uint32_t MB = PASS2 ? SP_MAXBINS2 : 256u;
    __shared__ uint32_t cnt[MB], lstart[MB], cursor[MB], delta[MB];
    __shared__ uint32_t wsum[SP_PART_BLOCK / 32];
    __shared__ __align__(8) uint64_t bars[SP_NBUF];
    __shared__ uint32_t rs_s, re_s, abort_s, group_s;
    const uint32_t tid = threadIdx.x;
    const uint32_t bins = PASS2 ? sp.bins2 : sp.bins1;
    if (PASS2 && !RESERVE && sp.bcap[0] != 0 && *(volatile const uint32_t*)sp.spill == 0) return;
    if (!PASS2 && sp.gate1 && *(volatile const uint32_t*)sp.gate1 == 0) return;
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < SP_NBUF; ++i) mbar_init(&bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK) cnt[d] = 0;
    // digit of a record: (cell >> (fs + shift)) & mask
    const uint32_t dshift = sp.fs + (PASS2 ? 0u : sp.hi_shift);
    const uint32_t mask = PASS2 ? sp.bins2 - 1 : 0xFFFFFFFFu;
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    // output slots: the records, or the reserved layout's slots (a run that
    // found its bucket full goes to n_slots, past the end, and is dropped)
    const uint32_t limit = RESERVE ? sp.n_slots : n_recs;
    const uint32_t lane = tid & 31u, w = tid >> 5;
    constexpr int IPT = SP_TILE / SP_PART_BLOCK;
    const uint32_t n_segs = PASS2 ? sp.nseg2_cap : sp.nseg1;
    // tiles this CTA has consumed before the current segment: tile g of the
    // CTA uses buffer g % SP_NBUF at barrier phase (g / SP_NBUF) & 1
    uint32_t g0 = 0;
    for (uint32_t seg = blockIdx.x; seg < n_segs; seg += gridDim.x) {
        __syncthreads();   // the previous segment's last tile is written out
        if (tid == 0) {
            uint32_t rs = 0, re = 0;
            if (PASS2) {
                const Seg2 sg = seg2_of(sp, seg);
                if (sg.valid) {
                    rs = sg.rs;
                    re = sg.re;
                    group_s = sg.group;
                }
            } else {
                const uint64_t nr = sp_records(sp);
                const uint64_t a = (uint64_t)seg * SP_SEGK * sp.n_tables;
                const uint64_t e = a + (uint64_t)SP_SEGK * sp.n_tables;
                rs = (uint32_t)(a < nr ? a : nr);
                re = (uint32_t)(e < nr ? e : nr);
            }
            rs_s = rs;
            re_s = re;
        }
        __syncthreads();
        const uint32_t rs = rs_s, re = re_s;
        if (rs >= re) continue;
        // segment cursors
        if (PASS2 && !RESERVE) {
            const Seg2 sg = seg2_of(sp, seg);
            const uint64_t base = (uint64_t)sp.bins2 * sp.plan[sg.group];
            for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK)
                cursor[d] = sp.off2[base + (uint64_t)d * sg.nseg + sg.k];
        } else if (!PASS2) {
            for (uint32_t d = tid; d < bins; d += SP_PART_BLOCK)
                cursor[d] = sp.off1[(uint64_t)d * sp.nseg1 + seg];
        }
        const uint32_t group = PASS2 ? group_s : 0u;
        const uint32_t n_tiles = (re - rs + SP_TILE - 1) / SP_TILE;
        // tile i covers records [rs + i*SP_TILE, ...); its copy starts at the
        // even index at or below, so the copy is 16-byte aligned and sized
        auto issue = [&](uint32_t i) {
            const uint32_t ts = rs + i * SP_TILE;
            const uint32_t te = ts + SP_TILE < re ? ts + SP_TILE : re;
            const uint32_t a0 = ts & ~1u, a1 = (te + 1) & ~1u;
            const uint32_t b = (g0 + i) % SP_NBUF;
            mbar_expect(&bars[b], (a1 - a0) * 8u);
            bulk_load(inbuf + b * SP_BUF, rin + a0, (a1 - a0) * 8u, &bars[b]);
        };
        if (tid == 0) {
            // the buffers' last readers (the previous segment) are past the barrier above
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (uint32_t i = 0; i < SP_NBUF && i < n_tiles; ++i) issue(i);
        }
        for (uint32_t i = 0; i < n_tiles; ++i) {
            const uint32_t gi = g0 + i;
            const uint32_t ts = rs + i * SP_TILE;
            const uint32_t nt = re - ts < SP_TILE ? re - ts : SP_TILE;
            const uint64_t* src = inbuf + (gi % SP_NBUF) * SP_BUF + (ts & 1u);
            // one thread waits for the tile's copy, the others at the barrier
            // (waiting warps would take issue slots from the working ones); the
            // barrier also orders the previous tile's reads of stage / delta
            // before this tile's writes
            if (tid == 0 && !copy_wait(sp, &bars[gi % SP_NBUF], (gi / SP_NBUF) & 1u)) abort_s = 1u;
            __syncthreads();
            if (abort_s) {
                // give the copies in flight a last bounded wait, then leave
                if (tid == 0) {
                    atomicOr(sp.err, GDBG_ERR_COPY_TIMEOUT);
                    for (uint32_t j = i; j < i + SP_NBUF && j < n_tiles; ++j)
                        mbar_wait(&bars[(g0 + j) % SP_NBUF], ((g0 + j) / SP_NBUF) & 1u);
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
            // reserved layout: the run's place is taken now, its latency
            // hidden behind the scan
            int rti = 0;
            uint32_t at = 0;
            if (RESERVE && c) {
                const uint32_t bk = (group << sp.hi_shift) | tid;
                while (rti + 1 < (int)sp.n_tables && sp.bbase[rti + 1] <= bk) ++rti;
                at = atomicAdd(sp.bfill + bk, c);
            }
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
                if (RESERVE) {
                    uint32_t dl = sp.n_slots;
                    if (c) {
                        const uint32_t bk = (group << sp.hi_shift) | tid;
                        if (at + c <= sp.bcap[rti])
                            dl = sp.cbase[rti] + (bk - sp.bbase[rti]) * sp.bcap[rti] + at - ex;
                        else
                            atomicExch(sp.spill, 1u);
                    }
                    delta[tid] = dl;
                } else {
                    delta[tid] = cursor[tid] - ex;
                    cursor[tid] += c;
                }
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
                    if (p < limit) rout[p] = v;
                    else if (!RESERVE) atomicOr(sp.err, GDBG_ERR_PARTITION);
                }
            }
        }
        g0 += n_tiles;
    }
}

// ---- 3d. bucket starts ---------------------------------------------------------

// First record of bucket bk in the counted layout (bk == n_buckets: the end).
__device__ __forceinline__ uint32_t sp_counted_start(const SortParams& sp, uint32_t bk,
                                                     uint32_t n_recs) {
    if (bk >= sp.n_buckets) return n_recs;
    if (sp.bins2 == 1) return sp.off1[(uint64_t)bk * sp.nseg1];
    const uint32_t* s0 = sp.plan;
    const uint32_t* D = sp.plan + 3 * (sp.bins1 + 1);
    const uint32_t g = bk >> sp.hi_shift, d = bk & (sp.bins2 - 1);
    const uint32_t nseg = s0[g + 1] - s0[g];
    return nseg ? sp.off2[(uint64_t)sp.bins2 * s0[g] + (uint64_t)d * nseg] : D[g];
}

// Record range [start, end) of every bucket, in whichever layout pass 2 made.
__global__ void k_sp_starts(SortParams sp, uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
    const uint32_t bk = blockIdx.x * blockDim.x + threadIdx.x;
    if (bk >= sp.n_buckets) return;
    if (sp.bcap[0] != 0 && *(volatile const uint32_t*)sp.spill == 0) {
        int ti = 0;
        while (ti + 1 < (int)sp.n_tables && sp.bbase[ti + 1] <= bk) ++ti;
        const uint32_t a = sp.cbase[ti] + (bk - sp.bbase[ti]) * sp.bcap[ti];
        start[bk] = a;
        end[bk] = a + sp.bfill[bk];
        return;
    }
    const uint32_t n_recs = (uint32_t)sp_records(sp);
    start[bk] = sp_counted_start(sp, bk, n_recs);
    end[bk] = sp_counted_start(sp, bk + 1, n_recs);
}

// ---- 4. order-independent apply -------------------------------------------

// Shared memory of the apply: the bucket's table region, a map of the zero
// cells its records touch, and dirty-sector bits.  The records are read from
// global memory once, by the threads, while the region's bulk copy is in
// flight; the kernel is issue-bound, so the launcher gives the map the
// shared memory that four CTAs per SM leave beside their regions.
//
// A cell that is not zero before the batch takes its records' saturating
// increments directly.  A cell that is zero stays zero while the records are
// read: the map counts its touches and keeps the smallest k-mer ordinal among
// them (its first toucher, so that k-mer is new), and the value, min(max,
// touches), is written after the last record.  Since no zero cell changes
// before then, the zero test of a record does not depend on which records ran
// first.
//
// Map entry: (smallest ordinal << 32) | (cell << SP_TOUCH_BITS) | touches
// (saturating); cells of a region are below 2^20.
constexpr uint32_t SP_TOUCH_BITS = 12;
constexpr uint32_t SP_TOUCH_MAX = (1u << SP_TOUCH_BITS) - 1u;
// Linear-probe limit of a map entry.  A map filled to half its slots needs
// about two probes; an insert that runs this long reports the map full (a
// fresh table can put nearly every cell of a region in it), and the zero
// cells are then redone in narrower cell ranges.
constexpr uint32_t SP_PROBE_CAP = 64;
constexpr int SP_APPLY_CTAS = 4;    // CTAs per SM the launcher sizes the map for
constexpr uint32_t SP_APPLY_U = 4;  // records each thread has in flight

// Shared-memory layout of k_sp_apply (byte offsets): region words (padded
// to 16 bytes), map slots, the list of created slots (16-bit, padded to 16
// bytes), dirty sector bits.
struct ApplyLayout {
    uint32_t map_off, list_off, dirty_off, total;
};
__host__ __device__ constexpr ApplyLayout sp_apply_layout(uint32_t region_words, uint32_t slots) {
    const uint32_t region_b = ((region_words + 3u) & ~3u) * 4u;
    const uint32_t list_b = ((slots * 2u) + 15u) & ~15u;
    const uint32_t dirty_b = (((region_words + 7u) / 8u + 31u) / 32u) * 4u;
    return ApplyLayout{region_b, region_b + slots * 8u, region_b + slots * 8u + list_b,
                       region_b + slots * 8u + list_b + dirty_b};
}
__host__ __device__ constexpr size_t sp_apply_smem(uint32_t region_words, uint32_t slots) {
    return sp_apply_layout(region_words, slots).total;
}

__device__ __forceinline__ uint32_t sp_home(uint32_t co, uint32_t slots) {
    return __umulhi(co * 0x9E3779B1u, slots);
}

// One touch of zero cell co by the k-mer with ordinal g; a new entry's slot
// goes on the created list.  False when the probe limit ran out (the map is
// too full).
__device__ __forceinline__ bool sp_touch(uint64_t* map, uint32_t slots, uint32_t co, uint32_t g,
                                         uint16_t* list, uint32_t* n_list) {
    const uint32_t key = co << SP_TOUCH_BITS;
    uint32_t sl = sp_home(co, slots);
    for (uint32_t it = 0; it < SP_PROBE_CAP; ++it) {
        uint64_t cur = map[sl];
        if (cur == SP_EMPTY) {
            cur = atomicCAS((unsigned long long*)(map + sl), SP_EMPTY,
                            ((uint64_t)g << 32) | key | 1u);
            if (cur == SP_EMPTY) {
                list[atomicAdd(n_list, 1u)] = (uint16_t)sl;
                return true;
            }
        }
        if (((uint32_t)cur & ~SP_TOUCH_MAX) == key) {
            // the cell's entry: one more touch, the smaller ordinal (every
            // failed swap means another touch of this cell went in)
            for (uint32_t t = 0; t < (1u << 20); ++t) {
                const uint32_t o = (uint32_t)(cur >> 32) < g ? (uint32_t)(cur >> 32) : g;
                const uint32_t n = (uint32_t)cur & SP_TOUCH_MAX;
                const uint64_t want = ((uint64_t)o << 32) | key | (n + (n < SP_TOUCH_MAX ? 1u : 0u));
                const uint64_t prev = atomicCAS((unsigned long long*)(map + sl), cur, want);
                if (prev == cur) break;
                cur = prev;
            }
            return true;
        }
        if (++sl == slots) sl = 0;
    }
    return false;
}

// One CTA per bucket.  Pass over the records: increments of cells that were
// not zero, touches of zero cells into the map; then each zero cell gets its
// value and its first toucher is flagged new.  When the zero cells overflow
// the map, they are redone in narrower cell ranges (the increments stand).
template <int STORAGE>
__global__ void __launch_bounds__(SP_APPLY_BLOCK, SP_APPLY_CTAS)
k_sp_apply(TableParams tp, SortParams sp, const uint64_t* __restrict__ recs,
           const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
           uint32_t* __restrict__ new_bits, unsigned long long* counters) {
    extern __shared__ __align__(128) unsigned char sbytes[];
    __shared__ uint32_t overflow, abort_s, n_list;
    __shared__ __align__(8) uint64_t bar;
    const uint32_t tid = threadIdx.x;
    const uint32_t bk = blockIdx.x;
    const uint32_t rs = start[bk], re = end[bk];
    if (rs >= re) return;
    int ti = 0;
    while (ti + 1 < tp.n && sp.bbase[ti + 1] <= bk) ++ti;
    const uint32_t region_cells = 1u << sp.fs;
    const uint32_t region_words = region_cells / cells_per_word<STORAGE>();
    const uint32_t region_sectors = (region_words + 7) / 8;
    const uint32_t slots = sp.map_slots;
    const ApplyLayout L = sp_apply_layout(region_words, slots);
    uint32_t* region = reinterpret_cast<uint32_t*>(sbytes);
    uint64_t* map = reinterpret_cast<uint64_t*>(sbytes + L.map_off);
    uint16_t* list = reinterpret_cast<uint16_t*>(sbytes + L.list_off);
    uint32_t* dirty = reinterpret_cast<uint32_t*>(sbytes + L.dirty_off);
    const uint64_t c0 = (uint64_t)(bk - sp.bbase[ti]) << sp.fs;
    const uint64_t w0 = c0 / cells_per_word<STORAGE>();
    uint32_t nw = region_words;
    if (w0 + nw > sp.twords[ti]) nw = (uint32_t)(sp.twords[ti] - w0);
    const uint32_t* gsrc = tp.words[ti] + w0;
    // the region by one bulk copy when it is a whole number of 16-byte units
    const bool bulk_region = ((w0 & 3u) == 0) && ((nw & 3u) == 0);
    const uint32_t n_recs = re - rs;
    const uint64_t* brec = recs + rs;
    // dense buckets write the whole region back; sparse ones their dirty sectors
    const bool track = n_recs < region_sectors;
    if (tid == 0) {
        abort_s = 0;
        overflow = 0;
        n_list = 0;
        if (bulk_region) {
            mbar_init(&bar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            mbar_expect(&bar, nw * 4u);
            bulk_load(region, gsrc, nw * 4u, &bar);
        }
    }
    if (!bulk_region)
        for (uint32_t k = tid; k < nw; k += SP_APPLY_BLOCK) region[k] = __ldcs(gsrc + k);
    if (track)
        for (uint32_t k = tid; k < (region_sectors + 31) / 32; k += SP_APPLY_BLOCK) dirty[k] = 0;
    for (uint32_t k = tid; k < slots; k += SP_APPLY_BLOCK) map[k] = SP_EMPTY;
    // the first records in flight while the region arrives
    uint64_t r[SP_APPLY_U];
#pragma unroll
    for (uint32_t u = 0; u < SP_APPLY_U; ++u) {
        const uint32_t k = tid + u * SP_APPLY_BLOCK;
        r[u] = k < n_recs ? __ldcs(brec + k) : 0ull;
    }
    // one thread waits for the region's copy, the others at the barrier
    // (waiting warps would take issue slots from the other CTAs' work)
    if (tid == 0 && bulk_region && !copy_wait(sp, &bar, 0)) abort_s = 1u;
    __syncthreads();
    if (abort_s) {
        if (tid == 0) {
            atomicOr(sp.err, GDBG_ERR_COPY_TIMEOUT);
            mbar_wait(&bar, 0);
        }
        return;
    }
    const uint32_t co_mask = region_cells - 1;
    auto mark = [&](uint32_t word) {
        const uint32_t sec = word >> 3;
        atomicOr(dirty + (sec >> 5), 1u << (sec & 31u));
    };
    // the pass over the records
    for (uint32_t k0 = 0; k0 < n_recs; k0 += SP_APPLY_U * SP_APPLY_BLOCK) {
        if (k0) {
#pragma unroll
            for (uint32_t u = 0; u < SP_APPLY_U; ++u) {
                const uint32_t k = k0 + tid + u * SP_APPLY_BLOCK;
                r[u] = k < n_recs ? __ldcs(brec + k) : 0ull;
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < SP_APPLY_U; ++u) {
            if (k0 + tid + u * SP_APPLY_BLOCK >= n_recs) break;
            const uint32_t co = (uint32_t)(r[u] >> 32) & co_mask;
            uint32_t word, shift;
            region_cell<STORAGE>(co, word, shift);
            uint32_t cur = region[word];
            if (cell_value<STORAGE>(cur, shift) != 0) {
                if (STORAGE != GDBG_BIT) {
                    for (int it = 0; it < (1 << 20); ++it) {
                        if (cell_value<STORAGE>(cur, shift) >= cell_max<STORAGE>()) break;
                        const uint32_t prev = atomicCAS(region + word, cur, cur + (1u << shift));
                        if (prev == cur) {
                            if (track) mark(word);
                            break;
                        }
                        cur = prev;
                    }
                }
            } else if (!*(volatile uint32_t*)&overflow) {
                if (!sp_touch(map, slots, co, (uint32_t)r[u], list, &n_list)) overflow = 1;
            }
        }
    }
    __syncthreads();
    unsigned long long occ = 0;
    // zero cells of the map: their values, and their first touchers flagged new
    auto settle = [&]() {
        const uint32_t nl = n_list;
        for (uint32_t i = tid; i < nl; i += SP_APPLY_BLOCK) {
            const uint64_t e = map[list[i]];
            const uint32_t co = (uint32_t)e >> SP_TOUCH_BITS;
            const uint32_t n = (uint32_t)e & SP_TOUCH_MAX;
            const uint32_t g = (uint32_t)(e >> 32);
            uint32_t word, shift;
            region_cell<STORAGE>(co, word, shift);
            atomicOr(region + word, (n < cell_max<STORAGE>() ? n : cell_max<STORAGE>()) << shift);
            if (track) mark(word);
            if (g < sp.kmer_cap) {
                atomicOr(new_bits + (g >> 5), 1u << (g & 31u));
                if (ti == 0) ++occ;
            }
        }
    };
    if (!overflow) {
        settle();
    } else {
        // zero cells by ranges [lo, lo + width): still zero, nothing of them
        // applied yet; a range whose zero cells overflow the map is redone
        // narrower
        uint32_t lo = 0, width = region_cells >> 1;
        int guard = 0;
        for (; lo < region_cells && guard < 4096; ++guard) {
            const uint32_t hi = lo + width < region_cells ? lo + width : region_cells;
            __syncthreads();   // everyone is done with the map
            for (uint32_t k = tid; k < slots; k += SP_APPLY_BLOCK) map[k] = SP_EMPTY;
            if (tid == 0) {
                overflow = 0;
                n_list = 0;
            }
            __syncthreads();
            for (uint32_t k0 = 0; k0 < n_recs; k0 += SP_APPLY_U * SP_APPLY_BLOCK) {
#pragma unroll
                for (uint32_t u = 0; u < SP_APPLY_U; ++u) {
                    const uint32_t k = k0 + tid + u * SP_APPLY_BLOCK;
                    r[u] = k < n_recs ? __ldg(brec + k) : 0ull;
                }
#pragma unroll
                for (uint32_t u = 0; u < SP_APPLY_U; ++u) {
                    if (k0 + tid + u * SP_APPLY_BLOCK >= n_recs) break;
                    const uint32_t co = (uint32_t)(r[u] >> 32) & co_mask;
                    if (co < lo || co >= hi) continue;
                    uint32_t word, shift;
                    region_cell<STORAGE>(co, word, shift);
                    if (cell_value<STORAGE>(region[word], shift) != 0) continue;
                    if (*(volatile uint32_t*)&overflow) continue;
                    if (!sp_touch(map, slots, co, (uint32_t)r[u], list, &n_list)) overflow = 1;
                }
            }
            __syncthreads();
            if (overflow && width > 1) {
                width >>= 1;
                continue;
            }
            settle();
            lo = hi;
        }
        if (lo < region_cells && tid == 0) atomicOr(sp.err, GDBG_ERR_CLAIMS_FULL);
    }
    __syncthreads();
    uint32_t* gdst = tp.words[ti] + w0;
    if (!track && bulk_region) {
        // a dense bucket: the whole region back by one bulk copy, which the
        // copy engine reads out of shared memory while the SM goes on
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile(
                "cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
                "r"(smem_addr(region)), "r"(nw * 4u)
                : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            // the CTA's shared memory stays until the copy has read it
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
        occ = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)occ);
        if ((tid & 31) == 0 && occ) atomicAdd(counters + 1, occ);
        return;
    }
    // write back the region: the dirty sectors of a sparse bucket (8 words
    // each), every sector otherwise
    for (uint32_t sec = tid; sec < region_sectors; sec += SP_APPLY_BLOCK) {
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
    if ((tid & 31) == 0 && occ) atomicAdd(counters + 1, occ);
}

}  // namespace gdbg
