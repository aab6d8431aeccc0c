// Kernel templates for the dBG hot path.  Each storage kind instantiates
// them in its own translation unit (gdbg_kernels_<kind>.cu) so the build
// compiles in parallel.
//
// Work mapping: the k-mers of a batch are flattened in read order (k-mer g of
// the batch is position g - kofs[r] of read r).  A thread owns a run of H
// consecutive k-mers; it seeds the rolling hash once and rolls through the
// run, re-seeding where a read ends.  Consecutive lanes own consecutive runs,
// so a warp reads one contiguous stretch of the packed base stream.
//
// Insert is two passes per window of k-mers:
//   probe  - read every touched cell (the state before the window), note the
//            cells that were zero, and record for each such cell the smallest
//            window ordinal that touches it (claims map);
//   commit - apply the inserts (atomicOr / saturating compare-and-swap) and
//            mark k-mer g new iff it is the first toucher of a cell that was
//            zero.  That is exactly when the reference's sequential insert
//            sees a zero cell for g (bitstorage.hh:195-219,
//            bytestorage.cc:60-113, nibblestorage.cc:60-100), because cells
//            only grow and every touch makes a cell non-zero.
// A window is small enough that the probe pass leaves its table sectors in
// L2 for the commit pass.
#pragma once
#include "gdbg_device.cuh"

namespace gdbg {

constexpr int BLOCK = 256;

template <int H>
struct Run {
    uint64_t h[H];
    uint64_t fw[H];
    uint64_t rc[H];
    uint32_t read[H];
    uint8_t front[H];
    uint8_t back[H];
    uint32_t valid;
};

// Read holding flattened k-mer g0: the largest r with kofs[r] <= g0, searched
// between the reads that hold the map tiles around g0.
// `total` is the device-side k-mer count (only tiles below it are mapped).
__device__ __forceinline__ uint64_t find_read(const BatchView& b, uint64_t g0, uint64_t total) {
    uint64_t tile = g0 / MAP_TILE;
    uint64_t n_tiles = (total + MAP_TILE - 1) / MAP_TILE;
    if (n_tiles > b.n_map_tiles) n_tiles = b.n_map_tiles;
    uint64_t lo = b.tile_read[tile];
    uint64_t hi = (tile + 1 < n_tiles) ? (uint64_t)b.tile_read[tile + 1] : b.n_reads - 1;
    while (lo < hi) {
        uint64_t mid = (lo + hi + 1) >> 1;
        if (__ldg(b.kofs + mid) <= g0) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Hashes of k-mers [g0, min(g0+H, gend)).  KEEP_ENDS also records the first
// and last base of each k-mer (for neighbour hashes).
template <bool CANON, int H, bool KEEP_ENDS>
__device__ __forceinline__ void make_run(const BatchView& b, const HashParams& hp,
                                         uint64_t g0, uint64_t gend, Run<H>& run) {
    run.valid = 0;
    // the device-side total bounds every index below, whatever the host passed
    const uint64_t total = __ldg(b.kofs + b.n_reads);
    if (gend > total) gend = total;
    if (gend > b.n_map_tiles * MAP_TILE) gend = b.n_map_tiles * MAP_TILE;
    if (g0 >= gend) return;
    uint64_t r = find_read(b, g0, total);
    uint64_t kbeg = __ldg(b.kofs + r), kend = __ldg(b.kofs + r + 1);
    uint64_t base = __ldg(b.offsets + r) + (g0 - kbeg);
    uint64_t fw, rc;
    BaseCursor cin, cout;
    cin.init(b.packed, base);
    cout.init(b.packed, base);
    const uint32_t K = hp.K;
    fw = 0; rc = 0;
    uint32_t last = 0;
    for (uint32_t i = 0; i < K; ++i) {
        uint32_t c = cin.next();
        fw = rotl1(fw) ^ sym(c);
        if (CANON) rc ^= rotl64(sym(3u - c), i);
        last = c;
    }
#pragma unroll
    for (int j = 0; j < H; ++j) {
        uint64_t g = g0 + j;
        if (g >= gend) break;
        if (j > 0) {
            if (g >= kend) {
                do { ++r; kbeg = kend; kend = __ldg(b.kofs + r + 1); } while (kend <= g);
                base = __ldg(b.offsets + r) + (g - kbeg);
                cin.init(b.packed, base);
                cout.init(b.packed, base);
                fw = 0; rc = 0;
                for (uint32_t i = 0; i < K; ++i) {
                    uint32_t c = cin.next();
                    fw = rotl1(fw) ^ sym(c);
                    if (CANON) rc ^= rotl64(sym(3u - c), i);
                    last = c;
                }
            } else {
                uint32_t out = cout.next();
                uint32_t in = cin.next();
                roll_right<CANON>(hp, out, in, fw, rc);
                last = in;
            }
        }
        run.h[j] = hash_value<CANON>(fw, rc);
        run.fw[j] = fw;
        run.rc[j] = CANON ? rc : 0;
        run.read[j] = (uint32_t)r;
        if (KEEP_ENDS) {
            run.front[j] = (uint8_t)base_at(b.packed, cout.pos);
            run.back[j] = (uint8_t)last;
        }
        run.valid |= 1u << j;
    }
}

template <int H>
__device__ __forceinline__ void hash_run(const uint64_t* __restrict__ hashes, uint64_t g0,
                                         uint64_t gend, Run<H>& run) {
    run.valid = 0;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        uint64_t g = g0 + j;
        if (g < gend) {
            run.h[j] = __ldg(hashes + g);
            run.read[j] = (uint32_t)g;
            run.valid |= 1u << j;
        }
    }
}

__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

// ---------------------------------------------------------------------------
// probe pass over the run of k-mers g0 .. g0+H-1
template <int STORAGE, int H, int NT>
__device__ __forceinline__ void probe_run(const TableParams& tp, const WindowParams& w,
                                          uint64_t g0, const Run<H>& run) {
    const int n = NT > 0 ? NT : tp.n;
    constexpr int TG = NT > 0 ? NT : 1;   // tables handled together
    uint32_t fresh[H];
#pragma unroll
    for (int j = 0; j < H; ++j) fresh[j] = 0;
    unsigned long long occupied = 0;

    for (int i0 = 0; i0 < n; i0 += TG) {
        uint32_t word[H][TG];
        uint32_t shift[H][TG];
        uint64_t bin[H][TG];
#pragma unroll
        for (int j = 0; j < H; ++j) {
#pragma unroll
            for (int t = 0; t < TG; ++t) {
                const int i = i0 + t;
                if (((run.valid >> j) & 1u) && i < n) {
                    bin[j][t] = fastmod(run.h[j], tp.p[i], tp.m[i]);
                    Cell c = cell_of<STORAGE>(tp, i, bin[j][t]);
                    shift[j][t] = c.shift;
                    word[j][t] = __ldcg(c.word);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < H; ++j) {
#pragma unroll
            for (int t = 0; t < TG; ++t) {
                const int i = i0 + t;
                if (((run.valid >> j) & 1u) && i < n) {
                    const uint64_t local = g0 + j - w.start;
                    if (STORAGE != GDBG_BIT) w.words[local * n + i] = word[j][t];
                    if (cell_value<STORAGE>(word[j][t], shift[j][t]) == 0) {
                        fresh[j] |= 1u << i;
                        uint64_t id = ((uint64_t)i << 32) | bin[j][t];
                        bool created = claim_min(w.claims, w.claims_mask, w.epoch, id,
                                                 (uint32_t)local, w.err);
                        if (created && i == 0) ++occupied;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < H; ++j)
        if ((run.valid >> j) & 1u) w.fresh[g0 + j - w.start] = fresh[j];
    warp_add(w.counters + 1, occupied);
}

template <int STORAGE, bool CANON, int H, int NT, bool FROM_HASHES>
__global__ void __launch_bounds__(BLOCK)
k_probe(BatchView b, const uint64_t* __restrict__ hashes, HashParams hp, TableParams tp,
        WindowParams w) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = w.start + tid * H;
    Run<H> run;
    if (FROM_HASHES) hash_run<H>(hashes, g0, w.end, run);
    else make_run<CANON, H, false>(b, hp, g0, w.end, run);
    probe_run<STORAGE, H, NT>(tp, w, g0, run);
}

// ---------------------------------------------------------------------------
// commit pass over the run of k-mers g0 .. g0+H-1
template <int STORAGE, int H, int NT>
__device__ __forceinline__ void commit_run(const TableParams& tp, const WindowParams& w,
                                           uint64_t g0, const Run<H>& run) {
    const int n = NT > 0 ? NT : tp.n;
    constexpr int TG = NT > 0 ? NT : 1;
    uint32_t fresh[H];
    uint32_t isnew = 0;
#pragma unroll
    for (int j = 0; j < H; ++j)
        fresh[j] = ((run.valid >> j) & 1u) ? __ldcg(w.fresh + (g0 + j - w.start)) : 0u;

    for (int i0 = 0; i0 < n; i0 += TG) {
#pragma unroll
        for (int j = 0; j < H; ++j) {
#pragma unroll
            for (int t = 0; t < TG; ++t) {
                const int i = i0 + t;
                if (((run.valid >> j) & 1u) && i < n) {
                    const uint64_t local = g0 + j - w.start;
                    uint64_t bin = fastmod(run.h[j], tp.p[i], tp.m[i]);
                    Cell c = cell_of<STORAGE>(tp, i, bin);
                    if (STORAGE == GDBG_BIT) {
                        atomicOr(c.word, 1u << c.shift);
                    } else {
                        sat_increment<STORAGE>(c.word, c.shift, __ldcg(w.words + local * n + i), w.err);
                    }
                    if ((fresh[j] >> i) & 1u) {
                        uint64_t id = ((uint64_t)i << 32) | bin;
                        if (claim_lookup(w.claims, w.claims_mask, w.epoch, id) == (uint32_t)local)
                            isnew |= 1u << j;
                    }
                }
            }
        }
    }
    // per-read new counts, one atomic per run of same-read k-mers
    unsigned long long total = 0;
    if (w.n_new) {
        uint32_t cur = 0xFFFFFFFFu;
        unsigned long long acc = 0;
#pragma unroll
        for (int j = 0; j < H; ++j) {
            if (!((run.valid >> j) & 1u)) continue;
            if (run.read[j] != cur) {
                if (acc) atomicAdd(w.n_new + cur, acc);
                cur = run.read[j];
                acc = 0;
            }
            acc += (isnew >> j) & 1u;
        }
        if (acc) atomicAdd(w.n_new + cur, acc);
    }
    total = __popc(isnew);
    warp_add(w.counters + 0, total);
}

template <int STORAGE, bool CANON, int H, int NT, bool FROM_HASHES>
__global__ void __launch_bounds__(BLOCK)
k_commit(BatchView b, const uint64_t* __restrict__ hashes, HashParams hp, TableParams tp,
         WindowParams w) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = w.start + tid * H;
    Run<H> run;
    if (FROM_HASHES) hash_run<H>(hashes, g0, w.end, run);
    else make_run<CANON, H, false>(b, hp, g0, w.end, run);
    commit_run<STORAGE, H, NT>(tp, w, g0, run);
}

// ---------------------------------------------------------------------------
// a window of at most SMALL_BLOCK * H k-mers in one block: the probe pass, a
// block barrier (the probe's global writes are visible to the whole block
// after it), then the commit pass on the same hashes -- one launch instead
// of two for a single read or a small chunk of reads
template <int STORAGE, bool CANON, int H, int NT, bool FROM_HASHES>
__global__ void __launch_bounds__(SMALL_BLOCK, 1)
k_insert_small(BatchView b, const uint64_t* __restrict__ hashes, HashParams hp, TableParams tp,
               WindowParams w) {
    const uint64_t g0 = w.start + (uint64_t)threadIdx.x * H;
    Run<H> run;
    if (FROM_HASHES) hash_run<H>(hashes, g0, w.end, run);
    else make_run<CANON, H, false>(b, hp, g0, w.end, run);
    probe_run<STORAGE, H, NT>(tp, w, g0, run);
    __syncthreads();
    commit_run<STORAGE, H, NT>(tp, w, g0, run);
}

// ---------------------------------------------------------------------------
// One read's insert in one CTA (insert_sequence, dbg.hh:249-265): chunks of
// the read's k-mers in order, one k-mer per thread.  Per chunk every thread
// hashes its k-mer and loads its cells (all tables at once); the cells that
// were zero go into a shared-memory map keyed by (table, cell) that keeps
// the smallest k-mer of the chunk touching each -- the one that sees it zero
// in the sequential loop, so that k-mer is new -- and then every cell takes
// its saturating increment.  The next chunk starts after the CTA barrier,
// with this chunk's increments in place.  No claims map in global memory:
// one round trip of loads and one of updates per chunk.  With `done`, the
// last word written is (seq << 32) | device status, which a caller can watch
// in host memory instead of synchronising the stream.
constexpr int READ_BLOCK = 512;
constexpr uint32_t READ_SLOTS = 4096;   // map slots: twice a chunk's records at most
constexpr int READ_MAXNT = 8;           // tables (more take the windowed insert)

__host__ __device__ constexpr size_t read_insert_smem() { return (size_t)READ_SLOTS * 12; }

template <int STORAGE, bool CANON>
__global__ void __launch_bounds__(READ_BLOCK, 1)
k_insert_read(BatchView b, HashParams hp, TableParams tp, uint64_t* n_new,
              unsigned long long* counters, uint32_t* err, uint64_t* done, uint32_t seq) {
    extern __shared__ __align__(16) uint64_t rkey[];   // (table << 56) | cell, all ones = empty
    uint32_t* rfirst = reinterpret_cast<uint32_t*>(rkey + READ_SLOTS);   // smallest k-mer per key
    __shared__ unsigned long long red_new[READ_BLOCK / 32], red_occ[READ_BLOCK / 32];
    // the chunk's bases, copied once from the packed read (which may be in
    // host memory) when they fit (k-mers of up to 256 bases)
    constexpr uint32_t RB_WORDS = (READ_BLOCK + 256) / 16 + 2;
    __shared__ uint32_t rbases[RB_WORDS];
    const uint32_t tid = threadIdx.x;
    const int n = tp.n;
    const uint32_t K = hp.K;
    const uint64_t nk = __ldg(b.kofs + 1) - __ldg(b.kofs);
    const uint64_t base = __ldg(b.offsets);
    // k-mers per chunk: the chunk's records (k-mers x tables) fill at most half the map
    const uint32_t chunk = READ_SLOTS / 2 / (uint32_t)n < READ_BLOCK ? READ_SLOTS / 2 / (uint32_t)n
                                                                     : READ_BLOCK;
    unsigned long long my_new = 0, my_occ = 0;
    for (uint64_t c0 = 0; c0 < nk; c0 += chunk) {
        const uint32_t ck = nk - c0 < chunk ? (uint32_t)(nk - c0) : chunk;   // k-mers of the chunk
        // map slots: a power of two at least twice the chunk's records
        uint32_t sbits = 6;
        while ((1u << sbits) < 2u * ck * (uint32_t)n && sbits < 12) ++sbits;
        const uint32_t nslots = 1u << sbits;
        for (uint32_t k = tid; k < nslots; k += READ_BLOCK) {
            rkey[k] = ~0ull;
            rfirst[k] = 0xFFFFFFFFu;
        }
        const uint64_t w0 = (base + c0) >> 4;
        const uint32_t nwords = (uint32_t)(((base + c0 + ck + K - 1 + 15) >> 4) - w0);
        const bool staged = nwords <= RB_WORDS;
        if (staged)
            for (uint32_t k = tid; k < nwords; k += READ_BLOCK) rbases[k] = __ldg(b.packed + w0 + k);
        __syncthreads();
        const uint64_t j = c0 + tid;
        const bool act = tid < chunk && j < nk;
        uint64_t cell[READ_MAXNT];
        uint32_t word[READ_MAXNT], shift[READ_MAXNT];
        uint32_t fresh = 0, slot_of[READ_MAXNT];
        if (act) {
            // the k-mer's hash from its K bases (the rolling state's closed form)
            uint64_t fw = 0, rc = 0;
            const uint32_t p0 = (uint32_t)((base + j) - (w0 << 4));   // first base in rbases
            for (uint32_t i = 0; i < K; ++i) {
                const uint32_t q = p0 + i;
                const uint32_t c = staged ? (rbases[q >> 4] >> ((q & 15u) << 1)) & 3u
                                          : base_at(b.packed, base + j + i);
                fw ^= rotl64(sym(c), (K - 1u - i) & 63u);
                if (CANON) rc ^= rotl64(sym(3u - c), i & 63u);
            }
            const uint64_t h = hash_value<CANON>(fw, rc);
#pragma unroll
            for (int i = 0; i < READ_MAXNT; ++i) {
                if (i >= n) break;
                cell[i] = fastmod(h, tp.p[i], tp.m[i]);
                const Cell cl = cell_of<STORAGE>(tp, i, cell[i]);
                shift[i] = cl.shift;
                word[i] = __ldcg(cl.word);
            }
#pragma unroll
            for (int i = 0; i < READ_MAXNT; ++i) {
                if (i >= n) break;
                if (cell_value<STORAGE>(word[i], shift[i]) != 0) continue;
                fresh |= 1u << i;
                const uint64_t key = ((uint64_t)i << 56) | cell[i];
                uint32_t sl = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - sbits));
                for (uint32_t it = 0; it < nslots; ++it) {
                    const uint64_t cur = atomicCAS((unsigned long long*)(rkey + sl), ~0ull, key);
                    if (cur == ~0ull || cur == key) break;
                    sl = (sl + 1) & (nslots - 1);
                }
                slot_of[i] = sl;
                atomicMin(rfirst + sl, tid);
            }
        }
        __syncthreads();
        if (act) {
            bool isnew = false;
#pragma unroll
            for (int i = 0; i < READ_MAXNT; ++i) {
                if (!((fresh >> i) & 1u)) continue;
                if (rfirst[slot_of[i]] == tid) {
                    isnew = true;
                    if (i == 0) ++my_occ;
                }
            }
            my_new += isnew;
#pragma unroll
            for (int i = 0; i < READ_MAXNT; ++i) {
                if (i >= n) break;
                const Cell cl = cell_of<STORAGE>(tp, i, cell[i]);
                if (STORAGE == GDBG_BIT) atomicOr(cl.word, 1u << cl.shift);
                else sat_increment<STORAGE>(cl.word, cl.shift, word[i], err);
            }
        }
        // this chunk's increments are in place before the next chunk's loads
        __threadfence_block();
        __syncthreads();
    }
    // the read's new k-mers and table 0's newly occupied cells
    for (int o = 16; o > 0; o >>= 1) {
        my_new += __shfl_xor_sync(0xFFFFFFFFu, my_new, o);
        my_occ += __shfl_xor_sync(0xFFFFFFFFu, my_occ, o);
    }
    if ((tid & 31) == 0) {
        red_new[tid >> 5] = my_new;
        red_occ[tid >> 5] = my_occ;
    }
    __syncthreads();
    if (tid == 0) {
        unsigned long long tn = 0, to = 0;
        for (int k = 0; k < READ_BLOCK / 32; ++k) {
            tn += red_new[k];
            to += red_occ[k];
        }
        // the only writer of the read's count (it may live in host memory)
        if (n_new) *n_new += tn;
        if (tn) atomicAdd(counters + 0, tn);
        if (to) atomicAdd(counters + 1, to);
        if (done) {
            // the caller's token with the device status word, after every
            // update of this insert is visible system-wide
            __threadfence_system();
            *(volatile uint64_t*)done = ((uint64_t)seq << 32) | *(volatile uint32_t*)err;
        }
    }
}

// ---------------------------------------------------------------------------
// query: Bit -> AND over tables (bitstorage.cc:87-100); Byte/Nibble -> min
// over tables capped at 255 / 15 (bytestorage.cc:116-139, nibblestorage.cc:112-130)
template <int STORAGE, bool CANON, int H, int NT, bool FROM_HASHES>
__global__ void __launch_bounds__(BLOCK)
k_query(BatchView b, const uint64_t* __restrict__ hashes, HashParams hp, TableParams tp,
        uint64_t n_total, int16_t* __restrict__ counts, uint64_t* __restrict__ values) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = tid * H;
    Run<H> run;
    if (FROM_HASHES) hash_run<H>(hashes, g0, n_total, run);
    else make_run<CANON, H, false>(b, hp, g0, n_total, run);
    const int n = NT > 0 ? NT : tp.n;
    constexpr int TG = NT > 0 ? NT : 1;
    uint32_t best[H];
#pragma unroll
    for (int j = 0; j < H; ++j) best[j] = cell_max<STORAGE>();
    for (int i0 = 0; i0 < n; i0 += TG) {
        uint32_t word[H][TG], shift[H][TG];
#pragma unroll
        for (int j = 0; j < H; ++j)
#pragma unroll
            for (int t = 0; t < TG; ++t) {
                const int i = i0 + t;
                if (((run.valid >> j) & 1u) && i < n) {
                    Cell c = cell_of<STORAGE>(tp, i, fastmod(run.h[j], tp.p[i], tp.m[i]));
                    shift[j][t] = c.shift;
                    word[j][t] = __ldcg(c.word);
                }
            }
#pragma unroll
        for (int j = 0; j < H; ++j)
#pragma unroll
            for (int t = 0; t < TG; ++t) {
                const int i = i0 + t;
                if (((run.valid >> j) & 1u) && i < n)
                    best[j] = min(best[j], cell_value<STORAGE>(word[j][t], shift[j][t]));
            }
    }
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (!((run.valid >> j) & 1u)) continue;
        counts[g0 + j] = (int16_t)best[j];
        if (values) values[g0 + j] = run.h[j];
    }
}

// ---------------------------------------------------------------------------
// hash values (and the fw / rc pair) of every k-mer
template <bool CANON, int H>
__global__ void __launch_bounds__(BLOCK)
k_hashes(BatchView b, HashParams hp, uint64_t* __restrict__ values, uint64_t* __restrict__ fw,
         uint64_t* __restrict__ rc) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = tid * H;
    Run<H> run;
    make_run<CANON, H, false>(b, hp, g0, b.n_kmers, run);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (!((run.valid >> j) & 1u)) continue;
        if (values) values[g0 + j] = run.h[j];
        if (fw) fw[g0 + j] = run.fw[j];
        if (rc) rc[g0 + j] = run.rc[j];
    }
}

// ---------------------------------------------------------------------------
// neighbour masks: the 4 left and 4 right extensions of every k-mer
// (hashextender.hh:352-396), each present iff every table cell is non-zero
// (query() != 0, unitig_walker.hh:361-372).
// SMALLP: every table is below 2^31 cells (32-bit remainders).
template <int STORAGE, bool CANON, int NT, bool SMALLP = false>
__device__ __forceinline__ bool present(const TableParams& tp, uint64_t h) {
    const int n = NT > 0 ? NT : tp.n;
    bool ok = true;
    if (NT > 0) {
        uint32_t word[NT > 0 ? NT : 1], shift[NT > 0 ? NT : 1];
#pragma unroll
        for (int i = 0; i < (NT > 0 ? NT : 1); ++i) {
            Cell c = cell_of<STORAGE>(tp, i, SMALLP ? (uint64_t)fastmod_small(h, (uint32_t)tp.p[i], tp.m[i])
                                                    : fastmod(h, tp.p[i], tp.m[i]));
            shift[i] = c.shift;
            word[i] = __ldcg(c.word);
        }
#pragma unroll
        for (int i = 0; i < (NT > 0 ? NT : 1); ++i)
            ok = ok && cell_value<STORAGE>(word[i], shift[i]) != 0;
    } else {
        for (int i = 0; i < n && ok; ++i) {
            Cell c = cell_of<STORAGE>(tp, i, fastmod(h, tp.p[i], tp.m[i]));
            ok = cell_value<STORAGE>(__ldcg(c.word), c.shift) != 0;
        }
    }
    return ok;
}

// Presence of 8 neighbour hashes as a bit mask (bit k = nh[k] present), for
// NT > 1 tables, in two rounds of independent loads: table 0 for every
// neighbour, then tables 1 .. NT-1 only for the neighbours whose table-0
// cell is set.  A neighbour is present iff all its cells are non-zero, as
// in present(); most absent neighbours are settled by their table-0 cell,
// and no neighbour's probes wait for another neighbour's.
template <int STORAGE, int NT, bool SMALLP>
__device__ __forceinline__ uint32_t neighbor_mask(const TableParams& tp, const uint64_t (&nh)[8]) {
    auto bin = [&](int i, uint64_t h) -> uint64_t {
        return SMALLP ? (uint64_t)fastmod_small(h, (uint32_t)tp.p[i], tp.m[i])
                      : fastmod(h, tp.p[i], tp.m[i]);
    };
    uint32_t cand = 0;
    {
        uint32_t w0[8], s0[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const Cell c = cell_of<STORAGE>(tp, 0, bin(0, nh[k]));
            w0[k] = __ldcg(c.word);
            s0[k] = c.shift;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (cell_value<STORAGE>(w0[k], s0[k]) != 0) cand |= 1u << k;
    }
    // the candidates' other cells, all loads issued before any is tested
    uint32_t w[8][NT - 1], s[8][NT - 1];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
#pragma unroll
        for (int i = 1; i < NT; ++i) {
            w[k][i - 1] = 0;
            s[k][i - 1] = 0;
            if ((cand >> k) & 1u) {
                const Cell c = cell_of<STORAGE>(tp, i, bin(i, nh[k]));
                w[k][i - 1] = __ldcg(c.word);
                s[k][i - 1] = c.shift;
            }
        }
    }
    uint32_t m = cand;
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int i = 1; i < NT; ++i)
            if (cell_value<STORAGE>(w[k][i - 1], s[k][i - 1]) == 0) m &= ~(1u << k);
    return m;
}

template <int STORAGE, bool CANON, int H, int NT, bool SMALLP>
__global__ void __launch_bounds__(BLOCK)
k_masks(BatchView b, HashParams hp, TableParams tp, uint8_t* __restrict__ masks) {
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t g0 = tid * H;
    Run<H> run;
    make_run<CANON, H, true>(b, hp, g0, b.n_kmers, run);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (!((run.valid >> j) & 1u)) continue;
        const uint64_t fw = run.fw[j], rc = run.rc[j];
        const uint32_t f = run.front[j], bk = run.back[j];
        uint64_t nh[8];
#pragma unroll
        for (uint32_t c = 0; c < 4; ++c) {
            uint64_t lf = fw, lr = rc;
            roll_left<CANON>(hp, c, bk, lf, lr);
            nh[c] = hash_value<CANON>(lf, lr);
            uint64_t rf = fw, rr = rc;
            roll_right<CANON>(hp, f, c, rf, rr);
            nh[4 + c] = hash_value<CANON>(rf, rr);
        }
        uint32_t m = 0;
        if constexpr (NT > 1) {
            m = neighbor_mask<STORAGE, NT, SMALLP>(tp, nh);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (present<STORAGE, CANON, NT, SMALLP>(tp, nh[k])) m |= 1u << k;
        }
        masks[g0 + j] = (uint8_t)m;
    }
}

}  // namespace gdbg
