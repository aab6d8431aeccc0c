// Parameter blocks shared by the host launchers and the kernels.
#pragma once
#include <cstdint>

#include "goetia_gb300.h"

namespace gdbg {

constexpr int MAX_TABLES = 32;

// Default poll limit of every bounded device wait (grid barrier, bulk-copy
// mbarrier): about a second or two of polling.
constexpr uint32_t WAIT_CAP = 1u << 24;

// Error bits accumulated in a device status word and surfaced by the C ABI.
enum : uint32_t {
    GDBG_ERR_CAS_LIMIT = 1u,      // a saturating compare-and-swap loop hit its cap
    GDBG_ERR_CLAIMS_FULL = 2u,    // the first-touch map overflowed
    GDBG_ERR_BARRIER_TIMEOUT = 4u,// a grid barrier wait hit its cap
    GDBG_ERR_BAD_OFFSETS = 8u,    // read offsets decrease or run past the packed stream
    GDBG_ERR_COPY_TIMEOUT = 16u,  // a bulk-copy wait hit its cap
    GDBG_ERR_PARTITION = 32u      // a partition position fell outside the record array
};

struct HashParams {
    uint64_t tk[4];   // rotl(T[c], K mod 64) for the four codes
    uint32_t K;
};

struct TableParams {
    uint32_t* words[MAX_TABLES];  // table i as 32-bit words
    uint64_t p[MAX_TABLES];       // table size (prime) in cells
    uint64_t m[MAX_TABLES];       // floor((2^64-1)/p)
    int n;
};

// A batch of reads already resident on the device.
struct BatchView {
    const uint32_t* packed;    // 2-bit base stream
    const uint64_t* offsets;   // n_reads+1 base offsets
    const uint64_t* kofs;      // n_reads+1 exclusive prefix of per-read k-mer counts
    const uint32_t* tile_read; // read holding k-mer t*MAP_TILE, per map tile
    uint64_t n_reads;
    uint64_t n_kmers;          // host copy of kofs[n_reads]
    uint64_t n_map_tiles;
    const uint64_t* tofs;      // n_reads+1 exclusive prefix of per-read warp tasks
    const uint32_t* task_read; // read of each warp task
    uint64_t task_cap;         // entries of task_read that are valid to read
};

constexpr uint64_t MAP_TILE = 1024;  // k-mers per entry of tile_read
constexpr uint32_t TASK_KMERS = 32;  // k-mers per warp task (one lane each)
constexpr int SMALL_BLOCK = 512;      // threads of the one-block insert of a small window

// One window of the insert: k-mers [start, end) of the batch.
struct WindowParams {
    uint64_t start, end;
    uint32_t* fresh;       // per k-mer: bit i set when table i's cell was zero
    uint32_t* words;       // per k-mer x table: word seen by the probe pass
    uint64_t* claims;      // first-touch map
    uint32_t claims_mask;
    uint32_t epoch;
    unsigned long long* n_new;   // per read (may be null)
    unsigned long long* counters;// [0] n_unique, [1] n_occupied
    uint32_t* err;
};

// Bucketed batch insert (gdbg_bucket.cuh).
constexpr int BK_BLOCK = 1024;        // threads per CTA in the bucket kernels
constexpr int BK_WARPS = BK_BLOCK / 32;
constexpr int BK_TPW = 2;             // warp tasks per warp per tile (k-mer passes)
constexpr int BK_RPW = 8;             // records per lane per tile (record passes)
constexpr int BK_MAXNT = 8;           // tables supported by the bucketed path
constexpr int BK_MAP = 2048;          // first-touch map slots per chunk (2 x block)

struct BucketParams {
    uint32_t fs;                      // log2(cells per bucket)
    uint32_t n_buckets;
    uint32_t shift;                   // digit position (in bucket-id bits) of this pass
    uint32_t n_tiles;
    uint64_t tbase[BK_MAXNT];         // aligned global cell base of each table
    uint32_t bbase[BK_MAXNT + 1];     // first bucket of each table
    uint32_t twords[BK_MAXNT];        // padded word count of each table
    const uint32_t* offsets;          // scatter: exclusive scan of hist (bin-major)
    uint32_t* hist;                   // histogram output (bin-major: bin * n_tiles + tile)
    const uint64_t* rin;
    uint64_t* rout;
    uint64_t n_recs;                  // host bound on the record count
    const uint64_t* total_kmers;      // device: the batch's k-mer count (kofs[n_reads])
    uint32_t n_tables;
    uint64_t kmer_cap;                // k-mers the new-k-mer bitmask can hold
};

// Segmented bucketed insert (gdbg_sort.cuh): records partitioned by bucket
// with two unstable most-significant-digit passes, then applied per bucket
// in an order-independent way.
constexpr uint32_t SP_TILE = 4096;       // records per partition tile
constexpr uint32_t SP_SEGK = 32768;      // k-mers per pass-1 segment (multiple of MAP_TILE)
constexpr uint32_t SP_SEG2 = 65536;      // records per pass-2 segment
constexpr uint32_t SP_MAXBINS2 = 512;    // pass-2 digit bins at most

struct SortParams {
    uint32_t fs;                  // log2(cells per bucket)
    uint32_t n_buckets;
    uint32_t n_tables;
    uint32_t hi_shift;            // pass-1 digit = bucket >> hi_shift
    uint32_t bins1, bins2;        // digit bins of pass 1 and pass 2 (bins2 == 1: one pass)
    uint64_t tbase[BK_MAXNT];     // aligned global cell base of each table
    uint32_t bbase[BK_MAXNT + 1]; // first bucket of each table
    uint32_t twords[BK_MAXNT];    // padded word count of each table
    const uint64_t* total_kmers;  // device: the batch's k-mer count
    uint64_t kmer_cap;            // host bound on k-mers
    uint32_t nseg1;               // pass-1 segments for kmer_cap k-mers
    uint32_t nseg2_cap;           // host bound on pass-2 segments
    uint32_t* hist1;              // bins1 x nseg1, bin-major
    uint32_t* off1;               // its exclusive scan
    uint32_t* hist2;              // ordered (group, bin, segment of the group)
    uint32_t* off2;               // its exclusive scan
    uint32_t* plan;               // s0[bins1 + 1] then G[bins1 + 1]
    uint32_t* err;                // device status word
    uint32_t wait_cap;            // polls of a bulk-copy wait before giving up (0: WAIT_CAP)
    uint32_t map_slots;           // apply: zero-cell map slots per CTA (set by its launcher)
    // Reserved layout of pass 2 (bcap[0] != 0): each bucket of table i owns
    // bcap[i] record slots from cbase[i] + (bucket - bbase[i]) * bcap[i] on,
    // and a pass-2 tile takes its runs' places by atomics on bfill; a bucket
    // that outgrows its slots sets *spill, and the counted, exact layout is
    // made instead.
    uint32_t bcap[BK_MAXNT];
    uint32_t cbase[BK_MAXNT];
    uint32_t n_slots;             // record slots of the pass-2 output
    uint32_t* bfill;              // records placed per bucket
    uint32_t* spill;
    // Reserved layout of pass 1 (gcap != nullptr: the emit and pass 1 fused,
    // k_sp_emit_part): digit group g owns gcap[g] slots from gbase[g] on;
    // lam[i] = records expected per bucket of table i (rounded up).  A group
    // that outgrows its slots sets *spill1, and the separate emit, its scan
    // and the counted pass 1 (gated on gate1 = spill1) make the exact layout.
    uint64_t lam[BK_MAXNT];
    uint32_t* gcap;
    uint32_t* gbase;
    uint32_t* gfill;
    uint32_t* spill1;
    const uint32_t* gate1;
    uint32_t n_slots1;            // record slots of the pass-1 output
};

// Persistent batch insert (gdbg_persist.cuh).
struct PersistParams {
    uint32_t window_tasks;        // warp tasks per window (<= 2^15)
    uint32_t* fresh;              // per window ordinal: zero-cell bits
    uint32_t* words;              // per window ordinal x table: word seen by the probe
    uint64_t* claims;
    uint32_t claims_mask;
    uint32_t* epoch_state;        // last claims epoch used (device, persists across calls)
    unsigned long long* n_new;    // per read, may be null
    unsigned long long* counters; // [0] n_unique, [1] n_occupied
    uint32_t* err;
    unsigned int* bar;            // [0] arrivals, [1] generation
    uint32_t spin_cap;            // polls of a grid-barrier wait before giving up (0: WAIT_CAP)
};

}  // namespace gdbg
