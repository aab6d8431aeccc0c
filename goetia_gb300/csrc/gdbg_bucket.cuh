// Bucketed insert for large batches on large tables.
//
// The per-k-mer insert touches 4 random table sectors per k-mer; once the
// tables are far larger than L2 every touch is a DRAM round trip and the DRAM
// traffic per k-mer is several times the algorithmic 256 bytes.  This path
// turns the batch's random updates into streams:
//
//   1. every k-mer g yields one record per table: (global cell id << 32) | g,
//      where the global cell id places table i at a base aligned to the
//      bucket size, and bucket = global cell id >> fs;
//   2. the records are stably partitioned by bucket with 8-bit digit passes
//      (per-warp histograms, bin-major scan, per-warp ranked scatter), so
//      inside a bucket they stay in ascending g;
//   3. one CTA per bucket loads the bucket's slice of its table into shared
//      memory, applies the records in chunks of the block size in g order and
//      writes the slice back.  Within a chunk, a k-mer is new on this table
//      when the cell is zero and no earlier record of the chunk touches the
//      same cell (a shared-memory min map); earlier chunks are already
//      applied.  That is the reference's sequential rule (bitstorage.hh:
//      195-219, bytestorage.cc:60-113, nibblestorage.cc:60-100) cell by cell;
//   4. new flags land in a per-k-mer bitmask; per-read counts are popcounts.
#pragma once
#include "gdbg_persist.cuh"

namespace gdbg {

// Records actually produced by the k-mer pass (device-side count, bounded by
// the host's allocation).
__device__ __forceinline__ uint64_t bk_records(const BucketParams& bp) {
    const uint64_t r = __ldg(bp.total_kmers) * bp.n_tables;
    return r < bp.n_recs ? r : bp.n_recs;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Lanes of the warp holding the same 8-bit digit (valid lanes only): one
// ballot per digit bit (warp multi-split).
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, bool valid) {
    uint32_t m = __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
    for (int bit = 0; bit < 8; ++bit) {
        const uint32_t vb = __ballot_sync(0xFFFFFFFFu, (d >> bit) & 1u);
        m &= ((d >> bit) & 1u) ? vb : ~vb;
    }
    return m;
}

// Position of this lane's record in the warp's running bin cursor, then
// advance the cursor by the group size.
__device__ __forceinline__ uint32_t warp_rank(uint32_t* row, uint32_t d, bool valid) {
    const uint32_t peers = digit_peers(d, valid);
    uint32_t pos = 0;
    if (valid) pos = row[d] + __popc(peers & lanemask_lt());
    __syncwarp();
    if (valid && (peers & lanemask_lt()) == 0) row[d] += __popc(peers);
    __syncwarp();
    return pos;
}

constexpr int BK_TB = 512;                    // threads per CTA, partition kernels
constexpr int BK_TW = BK_TB / 32;
constexpr int BK_IPT = 8;                     // records per thread per tile
constexpr int BK_TILE = BK_TB * BK_IPT;       // records per tile
constexpr int BK_EMIT_BLOCK = 256;

__device__ __forceinline__ uint32_t rec_digit(uint64_t rec, const BucketParams& bp) {
    return (((uint32_t)(rec >> 32) >> bp.fs) >> bp.shift) & 255u;
}
__device__ __forceinline__ uint32_t rec_bucket(uint64_t rec, uint32_t fs) {
    return (uint32_t)(rec >> 32) >> fs;
}

// Records in k-mer order: R0[g * n + i] = (global cell of table i << 32) | g.
// Each warp stages its task's records in shared memory and writes them as one
// contiguous run.
template <bool CANON>
__global__ void __launch_bounds__(BK_EMIT_BLOCK)
k_bkt_emit(BatchView b, HashParams hp, TableParams tp, BucketParams bp) {
    __shared__ uint64_t stage[BK_EMIT_BLOCK / 32][32 * BK_MAXNT];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t n_tasks = __ldg(b.tofs + b.n_reads);
    if (n_tasks > b.task_cap) n_tasks = b.task_cap;
    const uint32_t n = (uint32_t)tp.n;
    const uint64_t warp0 = ((uint64_t)blockIdx.x * BK_EMIT_BLOCK + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * BK_EMIT_BLOCK) >> 5;
    for (uint64_t t = warp0; t < n_tasks; t += n_warps) {
        const TaskInfo ti = task_info(b, t, lane);
        uint64_t fw, rc;
        task_hash<CANON>(b.packed, ti.b0, hp, ti.valid, lane, fw, rc);
        const uint32_t cnt = __popc(__ballot_sync(0xFFFFFFFFu, ti.valid));
        if (ti.valid) {
            const uint64_t h = hash_value<CANON>(fw, rc);
#pragma unroll
            for (int i = 0; i < BK_MAXNT; ++i) {
                if (i < (int)n) {
                    const uint64_t c = fastmod(h, tp.p[i], tp.m[i]);
                    stage[w][lane * n + i] = ((bp.tbase[i] + c) << 32) | (uint32_t)ti.g;
                }
            }
        }
        __syncwarp();
        const uint64_t g0 = __shfl_sync(0xFFFFFFFFu, ti.g, 0);
        uint64_t* dst = bp.rout + g0 * n;
        for (uint32_t k = lane; k < cnt * n; k += 32) dst[k] = stage[w][k];
        __syncwarp();
    }
}

// Per-tile digit histogram, bin-major: hist[bin * n_tiles + tile].
__global__ void __launch_bounds__(BK_TB, 3)
k_bkt_hist(BucketParams bp) {
    __shared__ uint32_t cnt[256];
    for (int k = threadIdx.x; k < 256; k += BK_TB) cnt[k] = 0;
    __syncthreads();
    const uint64_t n_recs = bk_records(bp);
    const uint64_t base = (uint64_t)blockIdx.x * BK_TILE;
    uint64_t rec[BK_IPT];
#pragma unroll
    for (int j = 0; j < BK_IPT; ++j) {
        const uint64_t k = base + (uint64_t)j * BK_TB + threadIdx.x;
        rec[j] = k < n_recs ? __ldcs(bp.rin + k) : 0;
    }
#pragma unroll
    for (int j = 0; j < BK_IPT; ++j) {
        const uint64_t k = base + (uint64_t)j * BK_TB + threadIdx.x;
        if (k < n_recs) atomicAdd(cnt + rec_digit(rec[j], bp), 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 256; k += BK_TB)
        bp.hist[(uint64_t)k * bp.n_tiles + blockIdx.x] = cnt[k];
}

// Exclusive scan of 256 values in shared memory by the first 256 threads
// (8 warps); all threads must call.
__device__ __forceinline__ void scan256(const uint32_t* in, uint32_t* out, uint32_t* wsum) {
    const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t v = 0, s = 0;
    if (t < 256) {
        v = in[t];
        s = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += y;
        }
        if (lane == 31) wsum[w] = s;
    }
    __syncthreads();
    if (t < 256) {
        uint32_t add = 0;
        for (uint32_t k = 0; k < w; ++k) add += wsum[k];
        out[t] = add + s - v;
    }
    __syncthreads();
}

// Stable scatter of one tile by digit: rank in shared memory (per-warp
// histograms keep warp order), then write each bin's run contiguously.  The
// last pass also records, per bucket, the smallest output position of its
// records (start[], pre-filled with 0xFFFFFFFF).
template <bool LAST>
__global__ void __launch_bounds__(BK_TB, 3)
k_bkt_scatter(BucketParams bp, uint32_t* __restrict__ start) {
    extern __shared__ uint64_t sh[];
    uint64_t* stage = sh;                                           // BK_TILE
    uint32_t(*whist)[256] = (uint32_t(*)[256])(sh + BK_TILE);       // BK_TW x 256
    uint32_t* bin_cnt = (uint32_t*)(sh + BK_TILE) + BK_TW * 256;
    uint32_t* bin_local = bin_cnt + 256;
    uint32_t* bin_global = bin_local + 256;
    uint32_t* wsum = bin_global + 256;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = lane; k < 256; k += 32) whist[w][k] = 0;
    __syncwarp();
    const uint64_t n_recs = bk_records(bp);
    const uint64_t tile_base = (uint64_t)blockIdx.x * BK_TILE;
    const uint64_t wbase = tile_base + (uint64_t)w * 32 * BK_IPT;
    uint64_t rec[BK_IPT];
#pragma unroll
    for (int j = 0; j < BK_IPT; ++j) {
        const uint64_t k = wbase + (uint64_t)j * 32 + lane;
        rec[j] = k < n_recs ? __ldcs(bp.rin + k) : 0;
    }
    // per-warp counts: one shared-memory atomic per record (ranks come later)
#pragma unroll
    for (int j = 0; j < BK_IPT; ++j) {
        const uint64_t k = wbase + (uint64_t)j * 32 + lane;
        if (k < n_recs) atomicAdd(&whist[w][rec_digit(rec[j], bp)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 256) {
        const uint32_t bin = threadIdx.x;
        uint32_t run = 0;
        for (int ww = 0; ww < BK_TW; ++ww) {
            const uint32_t c = whist[ww][bin];
            whist[ww][bin] = run;
            run += c;
        }
        bin_cnt[bin] = run;
        bin_global[bin] = bp.offsets[(uint64_t)bin * bp.n_tiles + blockIdx.x];
    }
    __syncthreads();
    scan256(bin_cnt, bin_local, wsum);
#pragma unroll
    for (int j = 0; j < BK_IPT; ++j) {
        const uint64_t k = wbase + (uint64_t)j * 32 + lane;
        const bool v = k < n_recs;
        const uint32_t d = rec_digit(rec[j], bp);
        const uint32_t pos = warp_rank(whist[w], d, v);
        if (v) stage[bin_local[d] + pos] = rec[j];
    }
    __syncthreads();
    const uint64_t left = n_recs > tile_base ? n_recs - tile_base : 0;
    const uint32_t n_tile = left < (uint64_t)BK_TILE ? (uint32_t)left : (uint32_t)BK_TILE;
    for (uint32_t k = threadIdx.x; k < n_tile; k += BK_TB) {
        const uint64_t r = stage[k];
        const uint32_t d = rec_digit(r, bp);
        const uint32_t gpos = bin_global[d] + (k - bin_local[d]);
        bp.rout[gpos] = r;
        if (LAST) {
            const uint32_t bk = rec_bucket(r, bp.fs);
            if (k == 0 || rec_bucket(stage[k - 1], bp.fs) != bk) atomicMin(start + bk, gpos);
        }
    }
}

constexpr size_t bk_scatter_smem() {
    return (size_t)BK_TILE * 8 + (size_t)BK_TW * 256 * 4 + 3 * 256 * 4 + 8 * 4;
}

// start[n_buckets] = record count; empty buckets take the next bucket's start.
__global__ void __launch_bounds__(1024)
k_bkt_starts_fix(BucketParams bp, uint32_t* __restrict__ start) {
    __shared__ uint32_t carry_s;
    const uint32_t nb = bp.n_buckets;
    if (threadIdx.x == 0) {
        start[nb] = (uint32_t)bk_records(bp);
        carry_s = start[nb];
    }
    __syncthreads();
    // reverse inclusive min-scan, 1024 entries at a time from the end
    for (int64_t hi = (int64_t)nb - 1; hi >= 0; hi -= 1024) {
        const int64_t i = hi - threadIdx.x;
        uint32_t v = i >= 0 ? start[i] : 0xFFFFFFFFu;
        const uint32_t lane = threadIdx.x & 31;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
            if (lane >= o) v = min(v, y);
        }
        __shared__ uint32_t wmin[32];
        if (lane == 31) wmin[threadIdx.x >> 5] = v;
        __syncthreads();
        uint32_t pre = carry_s;
        for (uint32_t k = 0; k < (threadIdx.x >> 5); ++k) pre = min(pre, wmin[k]);
        v = min(v, pre);
        if (i >= 0) start[i] = v;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = v;
        __syncthreads();
    }
}

constexpr int BK_RPT = 2;                         // records per thread per chunk
constexpr int BK_CHUNK = BK_BLOCK * BK_RPT;       // records per chunk
constexpr int BK_AMAP = 2 * BK_CHUNK;             // chunk map slots

// One CTA per bucket.  Dynamic shared memory: the bucket's table words, the
// chunk map (keys, then minimum chunk ranks) and a dirty bit per 32-byte
// sector of the slice.  Records are applied in chunks of BK_CHUNK in g order;
// only dirty sectors are written back.
//
// IQ (insert_and_query counts, bytestorage.cc:142-150): every record's cell
// goes into the chunk map, whose value is then the head of a list of the
// chunk's records on that cell; a record's rank is the number of list
// entries before it in g order.  Its table's value right after its own
// insert is min(max, value before the chunk + rank + 1), stored to
// vals[table * kmer_cap + g]; it is new when the value before was 0 and
// its rank is 0.
template <int STORAGE, bool IQ>
__global__ void __launch_bounds__(BK_BLOCK)
k_bkt_apply(TableParams tp, BucketParams bp, const uint64_t* __restrict__ recs,
            const uint32_t* __restrict__ start, uint32_t* __restrict__ new_bits,
            unsigned long long* counters, uint8_t* __restrict__ vals) {
    extern __shared__ uint32_t smem[];
    const uint32_t bk = blockIdx.x;
    const uint32_t rs = start[bk], re = start[bk + 1];
    if (rs == re) return;
    int ti = 0;
    while (ti + 1 < tp.n && bp.bbase[ti + 1] <= bk) ++ti;
    const uint32_t region_cells = 1u << bp.fs;
    const uint32_t region_words = region_cells / cells_per_word<STORAGE>();
    const uint32_t region_sectors = (region_words + 7) / 8;
    const uint64_t c0 = (uint64_t)(bk - bp.bbase[ti]) << bp.fs;
    const uint64_t w0 = c0 / cells_per_word<STORAGE>();
    uint32_t nw = region_words;
    if (w0 + nw > bp.twords[ti]) nw = (uint32_t)(bp.twords[ti] - w0);
    uint32_t* region = smem;
    uint32_t* mkey = smem + region_words;
    uint32_t* mval = mkey + BK_AMAP;
    uint32_t* dirty = mval + BK_AMAP;
    uint32_t* nxt = dirty + ((region_sectors + 31) / 32);   // IQ: list links per chunk record
    const uint32_t* gsrc = tp.words[ti] + w0;
    const bool vec = ((w0 & 3u) == 0) && ((nw & 3u) == 0);
    if (vec) {
        const uint4* s4 = reinterpret_cast<const uint4*>(gsrc);
        uint4* d4 = reinterpret_cast<uint4*>(region);
        const uint32_t n4 = nw >> 2;
        constexpr int V = 4;   // loads in flight per thread
        for (uint32_t k0 = threadIdx.x; k0 < n4; k0 += BK_BLOCK * V) {
            uint4 v[V];
#pragma unroll
            for (int j = 0; j < V; ++j)
                if (k0 + j * BK_BLOCK < n4) v[j] = __ldcs(s4 + k0 + j * BK_BLOCK);
#pragma unroll
            for (int j = 0; j < V; ++j)
                if (k0 + j * BK_BLOCK < n4) d4[k0 + j * BK_BLOCK] = v[j];
        }
    } else {
        for (uint32_t k = threadIdx.x; k < nw; k += BK_BLOCK) region[k] = __ldcs(gsrc + k);
    }
    for (uint32_t k = threadIdx.x; k < BK_AMAP; k += BK_BLOCK) mkey[k] = 0;
    for (uint32_t k = threadIdx.x; k < (region_sectors + 31) / 32; k += BK_BLOCK) dirty[k] = 0;
    __syncthreads();
    const uint32_t co_mask = region_cells - 1;
    unsigned long long occ = 0;
    uint64_t next[BK_RPT];
#pragma unroll
    for (int r = 0; r < BK_RPT; ++r) {
        const uint32_t k = rs + r * BK_BLOCK + threadIdx.x;
        next[r] = k < re ? __ldcs(recs + k) : 0;
    }
    for (uint32_t base = rs; base < re; base += BK_CHUNK) {
        uint32_t co[BK_RPT], g[BK_RPT], word[BK_RPT], shift[BK_RPT], slot[BK_RPT];
        uint32_t before[BK_RPT];
        bool active[BK_RPT], fresh[BK_RPT];
#pragma unroll
        for (int r = 0; r < BK_RPT; ++r) {
            const uint32_t idx = r * BK_BLOCK + threadIdx.x;
            const uint32_t k = base + idx;
            active[r] = k < re;
            const uint64_t rec = next[r];
            if (k + BK_CHUNK < re) next[r] = __ldcs(recs + k + BK_CHUNK);
            co[r] = (uint32_t)(rec >> 32) & co_mask;
            g[r] = (uint32_t)rec;
            region_cell<STORAGE>(co[r], word[r], shift[r]);
            before[r] = active[r] ? cell_value<STORAGE>(region[word[r]], shift[r]) : 1u;
            fresh[r] = active[r] && before[r] == 0;
            slot[r] = 0;
            if (IQ ? active[r] : fresh[r]) {
                // register the cell in the chunk map (rank order = g order)
                uint32_t sl = (co[r] * 0x9E3779B1u) >> (32 - 12);
                for (int it = 0; it < BK_AMAP; ++it) {
                    const uint32_t prev = atomicCAS(mkey + sl, 0u, co[r] + 1u);
                    if (prev == 0u) {
                        mval[sl] = 0xFFFFFFFFu;
                        break;
                    }
                    if (prev == co[r] + 1u) break;
                    sl = (sl + 1) & (BK_AMAP - 1);
                }
                slot[r] = sl;
            }
        }
        __syncthreads();
        uint32_t rank[BK_RPT];
        if (IQ) {
#pragma unroll
            for (int r = 0; r < BK_RPT; ++r)
                if (active[r]) {
                    const uint32_t idx = r * BK_BLOCK + threadIdx.x;
                    nxt[idx] = atomicExch(mval + slot[r], idx);
                }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < BK_RPT; ++r) {
                const uint32_t idx = r * BK_BLOCK + threadIdx.x;
                uint32_t n = 0;
                if (active[r]) {
                    uint32_t j = mval[slot[r]];
                    for (int it = 0; it < BK_CHUNK && j != 0xFFFFFFFFu; ++it) {
                        n += j < idx;
                        j = nxt[j];
                    }
                }
                rank[r] = n;
            }
        } else {
#pragma unroll
            for (int r = 0; r < BK_RPT; ++r)
                if (fresh[r]) atomicMin(mval + slot[r], r * BK_BLOCK + threadIdx.x);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < BK_RPT; ++r) {
            const bool isnew = IQ ? fresh[r] && rank[r] == 0
                                  : fresh[r] && mval[slot[r]] == r * BK_BLOCK + threadIdx.x;
            if (IQ && active[r] && g[r] < bp.kmer_cap) {
                const uint32_t v = min(before[r] + rank[r] + 1u, cell_max<STORAGE>());
                vals[(uint64_t)ti * bp.kmer_cap + g[r]] = (uint8_t)v;
            }
            if (active[r]) {
                bool changed = false;
                if (STORAGE == GDBG_BIT) {
                    if (fresh[r]) {
                        atomicOr(region + word[r], 1u << shift[r]);
                        changed = true;
                    }
                } else {
                    uint32_t cur = region[word[r]];
                    for (int it = 0; it < BK_CHUNK + 1; ++it) {
                        if (cell_value<STORAGE>(cur, shift[r]) >= cell_max<STORAGE>()) break;
                        const uint32_t prev = atomicCAS(region + word[r], cur, cur + (1u << shift[r]));
                        if (prev == cur) {
                            changed = true;
                            break;
                        }
                        cur = prev;
                    }
                }
                if (changed) {
                    const uint32_t sec = word[r] >> 3;
                    atomicOr(dirty + (sec >> 5), 1u << (sec & 31u));
                }
            }
            if (isnew && g[r] < bp.kmer_cap) {
                atomicOr(new_bits + (g[r] >> 5), 1u << (g[r] & 31u));
                if (ti == 0) ++occ;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < BK_RPT; ++r)
            if (IQ ? active[r] : fresh[r]) mkey[slot[r]] = 0;
        __syncthreads();
    }
    // write back the dirty 32-byte sectors (8 words each)
    uint32_t* gdst = tp.words[ti] + w0;
    for (uint32_t sec = threadIdx.x; sec < region_sectors; sec += BK_BLOCK) {
        if (!((dirty[sec >> 5] >> (sec & 31u)) & 1u)) continue;
        const uint32_t wb = sec * 8;
        if (vec && wb + 8 <= nw) {
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

__host__ __device__ constexpr size_t bk_apply_smem(uint32_t region_words, bool iq = false) {
    return (size_t)region_words * 4 + 2 * BK_AMAP * 4 + ((region_words + 7) / 8 + 31) / 32 * 4 +
           (iq ? (size_t)BK_CHUNK * 4 : 0);
}

// insert_and_query counts per k-mer (bytestorage.cc:142-150,
// nibblestorage.cc:103-109): 1 when the k-mer was new, else the minimum over
// the tables of the values right after its own insert; BitStorage always 1
// (bitstorage.cc:78-84).
__global__ void k_iq_counts(const uint8_t* __restrict__ vals, uint64_t cap, uint32_t n_tables,
                            const uint32_t* __restrict__ new_bits, const uint64_t* __restrict__ total,
                            int16_t* __restrict__ counts, bool presence) {
    const uint64_t n = min(*total, cap);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int16_t c = 1;
        if (!presence && !((__ldg(new_bits + (k >> 5)) >> (k & 31u)) & 1u)) {
            uint32_t m = 0xFFu;
            for (uint32_t t = 0; t < n_tables; ++t) m = min(m, (uint32_t)__ldg(vals + t * cap + k));
            c = (int16_t)m;
        }
        counts[k] = c;
    }
}

// Per-read new counts from the new-k-mer bitmask, plus the batch total.
__global__ void k_bkt_read_new(const uint64_t* __restrict__ kofs, uint64_t n_reads,
                               const uint32_t* __restrict__ new_bits,
                               unsigned long long* __restrict__ n_new,
                               unsigned long long* counters) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0;
    if (r < n_reads) {
        const uint64_t a = kofs[r], e = kofs[r + 1];
        for (uint64_t wd = a >> 5; (wd << 5) < e; ++wd) {
            uint32_t v = __ldg(new_bits + wd);
            const uint64_t lo = wd << 5;
            if (a > lo) v &= ~0u << (a - lo);
            if (e < lo + 32) v &= (1u << (e - lo)) - 1u;
            cnt += __popc(v);
        }
        if (n_new) n_new[r] = cnt;
    }
    const uint32_t s = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(counters + 0, (unsigned long long)s);
}

}  // namespace gdbg
