// The emit and pass 1 of the segmented insert in one kernel (four tables).
//
// k_sp_groups sizes the reserved pass-1 layout: digit group g (buckets
// g << hi_shift .. (g + 1) << hi_shift) owns gcap[g] record slots from
// gbase[g] on -- its expected records (the batch's k-mer bound times each
// of its buckets' share of their table), plus 1/64 of that, plus two tiles
// (sp_group_cap).
//
// k_sp_emit_part: one CTA of SP_EP_BLOCK threads per segment of SP_SEGK
// k-mers; thread t rolls the hash along the run of SP_EP_RUN consecutive
// k-mers from k-mer t * SP_EP_RUN of the segment (re-seeding at read
// starts, a lane entering a new read seeded by its whole warp).  Every
// SP_EP_STEPS steps of all threads make a tile of records, (global cell <<
// 32) | k-mer ordinal, four per k-mer, partitioned by the first digit like a
// pass-1 tile: each record ranked by a shared-memory atomic as it is made
// (it stays in registers), a block scan of the tile's counts, one atomic add
// per (tile, group) on the group's fill count for the run's place, the runs
// staged in shared memory and written out contiguously.  The records never
// go through HBM unpartitioned.  A group that outgrows its slots sets
// *spill1; then the separate emit, its counts and the counted pass 1,
// launched behind this kernel every time and idle otherwise, make the exact
// layout instead.
#pragma once

#include "gdbg_sort.cuh"

namespace gdbg {

constexpr int SP_EP_BLOCK = 512;
constexpr uint32_t SP_EP_RUN = SP_SEGK / SP_EP_BLOCK;                // k-mers per thread
constexpr uint32_t SP_EP_STEPS = SP_TILE / (4u * SP_EP_BLOCK);       // steps per tile
static_assert(SP_EP_RUN % SP_EP_STEPS == 0, "whole tiles per run");

__host__ __device__ constexpr size_t sp_ep_smem() { return (size_t)SP_TILE * 8; }

// One block of 256 threads: gcap / gbase of the 256 groups, fill counts and
// the spill word cleared.
__global__ void __launch_bounds__(256) k_sp_groups(SortParams sp) {
    __shared__ uint32_t ws[8];
    const uint32_t g = threadIdx.x, lane = g & 31, w = g >> 5;
    const uint32_t cap = (uint32_t)sp_group_cap(sp, g);
    uint32_t inc = cap;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    uint32_t add = 0;
    for (uint32_t k = 0; k < w; ++k) add += ws[k];
    sp.gcap[g] = cap;
    sp.gbase[g] = add + inc - cap;
    sp.gfill[g] = 0;
    if (g == 0) *sp.spill1 = 0;
}

template <bool CANON, bool SMALLP>
__global__ void __launch_bounds__(SP_EP_BLOCK, 2)
k_sp_emit_part(BatchView b, HashParams hp, TableParams tp, SortParams sp, uint64_t* __restrict__ rout,
               uint32_t seg0) {
    extern __shared__ __align__(16) uint64_t stage[];   // a tile's records, grouped by digit
    __shared__ uint32_t cnt[256], lstart[256], delta[256], gcap_s[256], gbase_s[256];
    __shared__ uint32_t wsum[SP_EP_BLOCK / 32];
    // roll terms by (out, in): fw ^= symk(out) ^ sym(in), rc ^= symk(3-in) ^ sym(3-out)
    __shared__ uint64_t roll_fw[16], roll_rc[16];
    const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t s = seg0 + blockIdx.x;   // launches may cover a range of segments
    for (uint32_t k = tid; k < 256; k += SP_EP_BLOCK) {
        cnt[k] = 0;
        gcap_s[k] = sp.gcap[k];
        gbase_s[k] = sp.gbase[k];
    }
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
    const uint32_t F = m / SP_EP_RUN, P = m % SP_EP_RUN;   // full runs, length of the partial one
    const uint32_t my_len = tid < F ? SP_EP_RUN : (tid == F ? P : 0u);
    uint64_t r = 0, kend = 0, fw = 0, rc = 0;
    uint32_t left = 0;   // k-mers of the current read from the current one on
    EmitCursor cin, cout;
    const uint32_t K = hp.K;
    if (my_len) {
        const uint64_t ga = gs + (uint64_t)tid * SP_EP_RUN;
        r = find_read(b, ga, total);
        kend = __ldg(b.kofs + r + 1);
        left = (uint32_t)(kend - ga);
        const uint64_t base = __ldg(b.offsets + r) + (ga - __ldg(b.kofs + r));
        cin.init(b.packed, base);
        cout.init(b.packed, base);
        for (uint32_t i = 0; i < K; ++i) {
            const uint32_t c = cin.next();
            fw = rotl1(fw) ^ sym(c);
            if (CANON) rc ^= rotl64(sym(3u - c), i);
        }
    }
    // ordinals are below 2^32
    const uint32_t g0 = (uint32_t)gs + tid * SP_EP_RUN;
    const uint32_t dsh = sp.fs + sp.hi_shift;   // first digit = cell >> dsh (dsh < 32)
    const uint32_t limit = sp.n_slots1;
    const uint32_t n_steps = F ? SP_EP_RUN : P;   // the longest run of the block
    constexpr int IPT = SP_TILE / SP_EP_BLOCK;
    for (uint32_t j0 = 0; j0 < n_steps; j0 += SP_EP_STEPS) {
        // the tile: steps j0 .. j0 + SP_EP_STEPS - 1 of every active thread,
        // four records per step; each record is ranked among the tile's
        // records of its digit as it is made (the rank and digit share a
        // word: digit < 2^8, rank < 2^13), and kept in registers
        uint32_t slot0 = 0;
        uint32_t cell[4 * SP_EP_STEPS], dp[4 * SP_EP_STEPS];
#pragma unroll
        for (uint32_t q = 0; q < SP_EP_STEPS; ++q) {
            const uint32_t j = j0 + q;
            const bool act = j < my_len;
            bool reseed = false;
            uint64_t rbase = 0;
            if (act && j > 0) {
                if (--left == 0) {
                    const uint64_t gk = gs + (uint64_t)tid * SP_EP_RUN + j;
                    do {
                        ++r;
                        kend = __ldg(b.kofs + r + 1);
                    } while (kend <= gk);
                    left = (uint32_t)(kend - gk);
                    rbase = __ldg(b.offsets + r) + (gk - __ldg(b.kofs + r));
                    reseed = true;
                } else {
                    const uint32_t out = cout.next();
                    const uint32_t in = cin.next();
                    fw = rotl1(fw) ^ roll_fw[out * 4u + in];
                    if (CANON) rc = rotr1(rc ^ roll_rc[out * 4u + in]);
                }
            }
            // lanes that entered a new read: the warp computes each one's seed
            // together, one base per lane, XOR-reduced
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
            const uint32_t A = j < P ? F + 1 : F;
            if (act) {
                const uint64_t h = hash_value<CANON>(fw, rc);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const uint32_t gc = (uint32_t)sp.tbase[i] +
                                        (SMALLP ? fastmod_small(h, (uint32_t)tp.p[i], tp.m[i])
                                                : (uint32_t)fastmod(h, tp.p[i], tp.m[i]));
                    const uint32_t d = gc >> dsh;
                    cell[4 * q + i] = gc;
                    dp[4 * q + i] = (atomicAdd(&cnt[d], 1u) << 8) | d;
                }
            }
            slot0 += A;
        }
        const uint32_t nt = slot0 * 4u;
        __syncthreads();
        // tile-local group starts (one group per thread), each run's place in
        // its group's slots
        const uint32_t c = tid < 256 ? cnt[tid] : 0u;
        if (tid < 256) cnt[tid] = 0;
        // the run's place in its group, taken now, its latency hidden behind the scan
        const uint32_t at = c ? atomicAdd(sp.gfill + tid, c) : 0u;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= (uint32_t)o) inc += y;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (tid < 256) {
            uint32_t pre = 0;
            for (uint32_t qq = 0; qq < w; ++qq) pre += wsum[qq];
            const uint32_t ex = pre + inc - c;
            lstart[tid] = ex;
            uint32_t dl = limit;   // a run that found its group full is dropped
            if (c) {
                if (at + c <= gcap_s[tid]) dl = gbase_s[tid] + at - ex;
                else atomicExch(sp.spill1, 1u);
            }
            delta[tid] = dl;
        }
        __syncthreads();
#pragma unroll
        for (uint32_t q = 0; q < SP_EP_STEPS; ++q) {
            if (j0 + q >= my_len) break;
            const uint64_t gl = g0 + j0 + q;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                stage[lstart[dp[4 * q + i] & 255u] + (dp[4 * q + i] >> 8)] =
                    ((uint64_t)cell[4 * q + i] << 32) | gl;
        }
        __syncthreads();
        // runs of equal digits go out contiguously
#pragma unroll
        for (int jj = 0; jj < IPT; ++jj) {
            const uint32_t k = jj * SP_EP_BLOCK + tid;
            if (k < nt) {
                const uint64_t v = stage[k];
                const uint32_t p = delta[(uint32_t)(v >> 32) >> dsh] + k;
                if (p < limit) rout[p] = v;
            }
        }
        __syncthreads();   // the tile and stage are free for the next steps
    }
}

}  // namespace gdbg
