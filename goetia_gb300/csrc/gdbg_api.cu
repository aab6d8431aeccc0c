// C ABI of the GB300 dBG hot path (declared in include/goetia_gb300.h).
//
// One gdbg_graph owns: the device tables (one allocation, each table padded
// to 256 bytes), its CUDA stream, the insert scratch (window buffers and the
// first-touch claims map), batch scratch (k-mer prefix, tile map) and
// staging buffers for the host-pointer entry points.  All device work of a
// handle runs on its stream in submission order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gdbg_device.cuh"
#include "gdbg_launch.h"
#include "goetia_gb300.h"

using namespace gdbg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define GDBG_CUDA(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(e_ == cudaErrorMemoryAllocation ? GDBG_ERR_OOM : GDBG_ERR_CUDA,      \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

#define GDBG_TRY(call)                       \
    do {                                     \
        int rc_ = (call);                    \
        if (rc_ != GDBG_OK) return rc_;      \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;  // elements
    int ensure(size_t n) {
        if (n <= cap) return GDBG_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(n + n / 4, 64);
        cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(GDBG_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        cap = want;
        return GDBG_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

uint32_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return (uint32_t)p;
}

}  // namespace

int gdbg::report_error(int code, const std::string& msg) { return fail(code, msg); }

// The storage proper: one device allocation holding every table (each padded
// to 256 bytes), the table sizes, the kernel-side table parameters and the
// n_unique / n_occupied counters.  Handles made by gdbg_share_storage point to
// the same store, the way dBGs built on one Storage share its shared_ptr
// (dbg.hh:97-101); it is freed with the last handle.
struct TableStore {
    int device = 0;
    std::vector<uint64_t> sizes, bytes, word_off, words;
    uint32_t* d_tables = nullptr;
    uint64_t total_words = 0;
    TableParams tp{};
    unsigned long long* d_counters = nullptr;  // [0] n_unique, [1] n_occupied
    ~TableStore() {
        cudaSetDevice(device);
        if (d_tables) cudaFree(d_tables);
        if (d_counters) cudaFree(d_counters);
    }
};

struct gdbg_graph {
    int storage = 0, shifter = 0;
    uint16_t K = 0;
    int device = 0;
    std::shared_ptr<TableStore> ts;   // tables and counters, shared by gdbg_share_storage
    HashParams hp{};
    cudaStream_t own_stream = nullptr, stream = nullptr;
    uint32_t* d_err = nullptr;
    // insert scratch
    uint32_t window = 262144, kpt = 4;
    DevBuf<uint32_t> fresh, words_seen;
    DevBuf<uint64_t> claims;
    uint32_t claims_mask = 0, epoch = 0;
    // persistent insert: device-owned claims epoch and grid-barrier state
    uint32_t pwindow = 262144;
    int path = GDBG_PATH_AUTO;
    bool persistent = true;
    // bucketed insert
    uint32_t bucket_fs = 0;   // 0 = default for the storage kind
    DevBuf<uint64_t> rec_a, rec_b;
    DevBuf<uint32_t> hist, hist_off, scan_parts, bstart, new_bits;
    DevBuf<uint8_t> iq_vals;    // insert_and_query: post-insert value per table and k-mer
    DevBuf<uint32_t> sp_hist2, sp_off2, sp_plan;   // segmented path: pass-2 counts, plan
    DevBuf<uint32_t> sp_fill, sp_end;              // spill word + per-bucket fill; bucket ends
    DevBuf<uint32_t> sp_groups;                    // fused pass 1: group slots, bases, fills, spill
    DevBuf<uint64_t> cq_keys;                      // compactor query: per-read new-k-mer sets
    DevBuf<uint32_t> cq_min, cq_ones;
    uint32_t* d_epoch = nullptr;
    unsigned int* d_bar = nullptr;
    // poll limits of the bounded device waits (0: the kernels' default)
    uint32_t barrier_polls = 0, copy_polls = 0;
    bool epoch_on_device = false;
    uint32_t epoch_staging = 0;
    // batch scratch
    DevBuf<uint64_t> kofs, tofs, partials;
    DevBuf<uint32_t> tile_read, task_read;
    // one-sequence calls: the read, its prefix and its maps built on the host
    // in one pinned block and moved by one copy; small results come back
    // through the pinned ret block
    // (mapped into the device's address space: insert_sequence's read kernel
    // reads the block in place and writes its count and status back into it)
    uint8_t* h_single = nullptr;
    uint8_t* h_single_dev = nullptr;     // the block's device address
    size_t h_single_cap = 0;
    DevBuf<uint8_t> d_single;
    cudaEvent_t single_done = nullptr;   // the last copy out of h_single
    uint64_t* single_nnew = nullptr;     // device n_new slot of the staged read
    bool read_smem_set = false;          // the read kernel's shared-memory opt-in is done
    uint32_t read_seq = 0;               // token of the last read insert watched in host memory
    struct Ret {
        uint32_t err, pad;
        uint64_t v[7];
    }* h_ret = nullptr;
    // host batch inserts: the packed reads move in chunks of whole reads on
    // copy_stream (chunk_ev[c] after chunk c) while the segmented emit runs on
    // the segments of the chunks already in; plan.kmer_end[c] is the k-mer
    // count of chunks 0..c (plan.n chunks, 0 when no plan is pending)
    static constexpr int N_CHUNKS = 4;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_ev[N_CHUNKS] = {}, prior_ev = nullptr;
    struct ChunkPlan {
        int n = 0;
        uint64_t kmer_end[N_CHUNKS];
    } plan;
    // asynchronous host-buffer inserts of large batches: two staging slots
    // used in turn, each filled on copy_stream while the batch before it
    // runs; `released` follows the last work that reads the slot
    static constexpr uint64_t ASYNC_SLOT_WORDS = 1u << 20;   // packed words (16 Mbp) and up
    struct AsyncSlot {
        DevBuf<uint32_t> packed;
        DevBuf<uint64_t> offsets, out;
        cudaEvent_t copied = nullptr, released = nullptr;
        bool pending = false;
    } aslot[2];
    int aslot_next = 0;
    // staging for host-pointer calls
    DevBuf<uint32_t> st_packed;
    DevBuf<uint64_t> st_offsets, st_out64, st_out64b, st_out64c;
    DevBuf<int16_t> st_counts;
    DevBuf<uint8_t> st_u8;
    uint64_t launches = 0;
    // optional per-stage timing (CUDA events around each stage, on its stream)
    bool profiling = false;
    struct Pending { const char* name; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> free_events;
    std::vector<std::pair<std::string, std::pair<double, uint64_t>>> stage_acc;

    LaunchShape shape(int kpt_) const {
        return LaunchShape{shifter == GDBG_CAN_LEMIRE, kpt_, (int)ts->sizes.size()};
    }
};

namespace {

cudaEvent_t take_event(gdbg_graph* g) {
    if (!g->free_events.empty()) {
        cudaEvent_t e = g->free_events.back();
        g->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Records a CUDA event pair around one stage when profiling is on.
struct Stage {
    gdbg_graph* g;
    const char* name;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    Stage(gdbg_graph* g_, const char* n, cudaStream_t s) : g(g_), name(n), st(s) {
        if (g->profiling) {
            a = take_event(g);
            cudaEventRecord(a, st);
        }
    }
    ~Stage() {
        if (a) {
            cudaEvent_t b = take_event(g);
            cudaEventRecord(b, st);
            g->pending.push_back({name, a, b});
        }
    }
};

// Resolve recorded stage events into the per-stage totals.
void collect_stages(gdbg_graph* g) {
    for (auto& p : g->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            bool found = false;
            for (auto& acc : g->stage_acc)
                if (acc.first == p.name) {
                    acc.second.first += ms;
                    acc.second.second += 1;
                    found = true;
                }
            if (!found) g->stage_acc.push_back({p.name, {ms, 1}});
        }
        g->free_events.push_back(p.a);
        g->free_events.push_back(p.b);
    }
    g->pending.clear();
}

int set_device(const gdbg_graph* g) {
    GDBG_CUDA(cudaSetDevice(g->device));
    return GDBG_OK;
}

cudaStream_t pick_stream(gdbg_graph* g, void* s) {
    return s ? (cudaStream_t)s : g->stream;
}

// Table layout in the single device allocation: table i holds its reference
// byte length (size/8+1, size, size/2+1 for Bit, Byte, Nibble) padded up to
// 256 bytes, at word offset word_off[i].  Returns the total in 32-bit words.
uint64_t table_layout(int storage, const uint64_t* sizes, uint16_t n, std::vector<uint64_t>& sz,
                      std::vector<uint64_t>& bytes, std::vector<uint64_t>& words,
                      std::vector<uint64_t>& word_off) {
    sz.clear(); bytes.clear(); words.clear(); word_off.clear();
    uint64_t off = 0;
    for (uint16_t i = 0; i < n; ++i) {
        uint64_t p = sizes[i];
        uint64_t b = storage == GDBG_BIT ? p / 8 + 1 : storage == GDBG_NIBBLE ? p / 2 + 1 : p;
        uint64_t w = ((b + 3) / 4 + 63) / 64 * 64;
        sz.push_back(p);
        bytes.push_back(b);
        words.push_back(w);
        word_off.push_back(off);
        off += w;
    }
    return off;
}

// Kernel-side table parameters (base pointers, sizes, fastmod magics).
void set_table_params(gdbg_graph* g) {
    const size_t n = g->ts->sizes.size();
    for (size_t i = 0; i < n; ++i) {
        g->ts->tp.words[i] = g->ts->d_tables + g->ts->word_off[i];
        g->ts->tp.p[i] = g->ts->sizes[i];
        g->ts->tp.m[i] = ~0ull / g->ts->sizes[i];
    }
    g->ts->tp.n = (int)n;
}

// Per-handle state: stream, status word, claims epoch, grid barrier and the
// hash constants for K.  The tables come from g->ts.
int init_handle(gdbg_graph* g, int storage, int shifter, uint16_t K) {
    g->storage = storage;
    g->shifter = shifter;
    g->K = K;
    if (cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(GDBG_ERR_CUDA, "cudaStreamCreate failed");
    g->stream = g->own_stream;
    // d_err[0]: device status bits; d_err[1]: offset check of a host batch
    if (cudaMalloc((void**)&g->d_err, 2 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&g->d_epoch, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&g->d_bar, 2 * sizeof(unsigned int)) != cudaSuccess)
        return fail(GDBG_ERR_OOM, "counter allocation failed");
    cudaMemsetAsync(g->d_epoch, 0, sizeof(uint32_t), g->stream);
    cudaMemsetAsync(g->d_bar, 0, 2 * sizeof(unsigned int), g->stream);
    cudaMemsetAsync(g->d_err, 0, 2 * sizeof(uint32_t), g->stream);
    if (cudaHostAlloc((void**)&g->h_ret, sizeof(gdbg_graph::Ret), cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->single_done, cudaEventDisableTiming) != cudaSuccess)
        return fail(GDBG_ERR_OOM, "pinned status allocation failed");
    g->hp = make_hash_params(K);
    return GDBG_OK;
}

int check_kinds(int storage, int shifter, uint16_t K) {
    if (storage < GDBG_BIT || storage > GDBG_NIBBLE)
        return fail(GDBG_ERR_INVALID_ARG, "unknown storage kind");
    if (shifter != GDBG_FWD_LEMIRE && shifter != GDBG_CAN_LEMIRE)
        return fail(GDBG_ERR_INVALID_ARG, "unknown shifter kind");
    if (K == 0) return fail(GDBG_ERR_INVALID_ARG, "K must be positive");
    return GDBG_OK;
}

int make_graph(int storage, int shifter, uint16_t K, const uint64_t* sizes, uint16_t n,
               gdbg_graph** out) {
    if (!out) return fail(GDBG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    GDBG_TRY(check_kinds(storage, shifter, K));
    if (n == 0 || n > MAX_TABLES)
        return fail(GDBG_ERR_INVALID_ARG, "n_tables must be in 1..32");
    for (uint16_t i = 0; i < n; ++i)
        if (sizes[i] == 0 || sizes[i] >= (1ull << 32))
            return fail(GDBG_ERR_INVALID_ARG, "table sizes must be in 1..2^32-1 cells");

    gdbg_graph* g = new gdbg_graph();
    cudaGetDevice(&g->device);
    g->ts = std::make_shared<TableStore>();
    g->ts->device = g->device;
    auto cleanup = [&](int rc) { gdbg_destroy(g); return rc; };
    const int rc = init_handle(g, storage, shifter, K);
    if (rc != GDBG_OK) return cleanup(rc);
    const uint64_t off = table_layout(storage, sizes, n, g->ts->sizes, g->ts->bytes, g->ts->words, g->ts->word_off);
    g->ts->total_words = off;
    cudaError_t e = cudaMalloc((void**)&g->ts->d_tables, off * sizeof(uint32_t));
    if (e != cudaSuccess) {
        g->ts->d_tables = nullptr;
        return cleanup(fail(GDBG_ERR_OOM, std::string("table allocation: ") + cudaGetErrorString(e)));
    }
    if (cudaMalloc((void**)&g->ts->d_counters, 2 * sizeof(unsigned long long)) != cudaSuccess)
        return cleanup(fail(GDBG_ERR_OOM, "counter allocation failed"));
    cudaMemsetAsync(g->ts->d_tables, 0, off * sizeof(uint32_t), g->stream);
    cudaMemsetAsync(g->ts->d_counters, 0, 2 * sizeof(unsigned long long), g->stream);
    set_table_params(g);
    e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cleanup(fail(GDBG_ERR_CUDA, cudaGetErrorString(e)));
    *out = g;
    return GDBG_OK;
}

// A non-zero device status word: cleared on the device, reported.
int device_status_fail(gdbg_graph* g, uint32_t err) {
    cudaMemsetAsync(g->d_err, 0, sizeof(uint32_t), g->stream);
    char buf[200];
    std::snprintf(buf, sizeof buf,
                  "device status 0x%x (1=CAS cap, 2=claims map full, 4=barrier timeout, "
                  "8=bad read offsets, 16=bulk-copy timeout, 32=partition overflow)", err);
    return fail(GDBG_ERR_DEVICE, buf);
}

int check_device_status(gdbg_graph* g) {
    GDBG_CUDA(cudaMemcpyAsync(&g->h_ret->err, g->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    const uint32_t err = g->h_ret->err;
    return err ? device_status_fail(g, err) : GDBG_OK;
}

// Per-read k-mer prefix + tile map for a device-resident batch.
// MAP_FOR_INSERT: the maps the insert path chosen for the batch's total needs
enum MapNeed { MAP_TILES = 1, MAP_TASKS = 2, MAP_FOR_INSERT = 4 };
int insert_maps(const gdbg_graph* g, uint64_t n_total);

// checked: the offsets came from a host batch and are validated by the prefix
// kernel into their own status word; with hint UINT64_MAX that word comes back
// with the total, so a bad batch fails before any table is touched.
// probe_reads: reads whose k-mer prefix kofs[r] comes back with the total
// (into probe_kofs; only with hint UINT64_MAX).
int prepare_batch(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                  const uint64_t* offsets, uint64_t n_reads, uint64_t hint, cudaStream_t st,
                  BatchView* view, int maps = MAP_TILES | MAP_TASKS, bool checked = false,
                  const uint64_t* probe_reads = nullptr, uint64_t* probe_kofs = nullptr,
                  int n_probe = 0) {
    GDBG_TRY(g->kofs.ensure(n_reads + 1));
    GDBG_TRY(g->tofs.ensure(n_reads + 1));
    GDBG_TRY(g->partials.ensure(2 * (n_reads / 1024 + 2)));
    int nl = 0;
    Stage stage_prep(g, "prepare", st);
    uint32_t* perr = checked ? g->d_err + 1 : g->d_err;
    if (checked) GDBG_CUDA(cudaMemsetAsync(perr, 0, sizeof(uint32_t), st));
    GDBG_CUDA(launch_kmer_prefix(offsets, n_reads, g->K, packed_words * 16ull, g->partials.p,
                                 g->kofs.p, g->tofs.p, perr, st, &nl));
    g->launches += nl;
    uint64_t total = hint, tasks = 0;
    if (total == UINT64_MAX) {
        // read back through the pinned block: [0] total, [1] tasks, [2] the
        // offset check, [3..] the probed prefixes
        uint64_t* tt = g->h_ret->v;
        if (n_probe > 4) n_probe = 4;
        tt[2] = 0;
        GDBG_CUDA(cudaMemcpyAsync(&tt[0], g->kofs.p + n_reads, sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, st));
        GDBG_CUDA(cudaMemcpyAsync(&tt[1], g->tofs.p + n_reads, sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, st));
        if (checked)
            GDBG_CUDA(cudaMemcpyAsync(&tt[2], perr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        for (int i = 0; i < n_probe; ++i)
            GDBG_CUDA(cudaMemcpyAsync(&tt[3 + i], g->kofs.p + probe_reads[i], sizeof(uint64_t),
                                      cudaMemcpyDeviceToHost, st));
        GDBG_CUDA(cudaStreamSynchronize(st));
        if (tt[2])
            return fail(GDBG_ERR_INVALID_ARG,
                        "offsets must be non-decreasing and end within the packed stream");
        total = tt[0];
        tasks = tt[1];
        for (int i = 0; i < n_probe; ++i) probe_kofs[i] = tt[3 + i];
    } else {
        // every read adds at most one partly filled task
        tasks = total / TASK_KMERS + std::min<uint64_t>(n_reads, total);
    }
    if (maps & MAP_FOR_INSERT) maps = insert_maps(g, total);
    uint64_t tiles = (total + MAP_TILE - 1) / MAP_TILE;
    GDBG_TRY(g->tile_read.ensure(tiles + 1));
    GDBG_TRY(g->task_read.ensure(tasks + 1));
    if (total) {
        if (maps & MAP_TILES) {
            GDBG_CUDA(launch_tile_map(g->kofs.p, n_reads, tiles, g->tile_read.p, st));
            g->launches += 1;
        }
        if (maps & MAP_TASKS) {
            GDBG_CUDA(launch_task_map(g->tofs.p, n_reads, tasks, g->task_read.p, st));
            g->launches += 1;
        }
    }
    view->packed = packed;
    view->offsets = offsets;
    view->kofs = g->kofs.p;
    view->tile_read = g->tile_read.p;
    view->n_reads = n_reads;
    view->n_kmers = total;
    view->n_map_tiles = tiles;
    view->tofs = g->tofs.p;
    view->task_read = g->task_read.p;
    view->task_cap = tasks;
    return GDBG_OK;
}

int ensure_insert_scratch(gdbg_graph* g, cudaStream_t st) {
    const uint64_t W = g->window, n = g->ts->sizes.size();
    GDBG_TRY(g->fresh.ensure(W));
    if (g->storage != GDBG_BIT) GDBG_TRY(g->words_seen.ensure(W * n));
    uint32_t slots = next_pow2(2 * W * n);
    if (g->claims.cap < slots) {
        g->claims.release();
        GDBG_TRY(g->claims.ensure(slots));
        GDBG_CUDA(cudaMemsetAsync(g->claims.p, 0, g->claims.cap * sizeof(uint64_t), st));
        g->epoch = 0;
    }
    g->claims_mask = slots - 1;
    return GDBG_OK;
}

int next_epoch(gdbg_graph* g, cudaStream_t st) {
    // epochs 1..127; slot value 0 (epoch 0) means empty
    if (g->epoch >= 127) {
        GDBG_CUDA(cudaMemsetAsync(g->claims.p, 0, g->claims.cap * sizeof(uint64_t), st));
        g->epoch = 0;
    }
    ++g->epoch;
    return GDBG_OK;
}

int launch_pass(gdbg_graph* g, int pass, const LaunchShape& s, uint64_t n_threads, cudaStream_t st,
                const BatchView& b, const uint64_t* hashes, const WindowParams& w) {
    cudaError_t e;
    switch (g->storage) {
    case GDBG_BIT: e = launch_insert_pass<GDBG_BIT>(pass, s, n_threads, st, b, hashes, g->hp, g->ts->tp, w); break;
    case GDBG_BYTE: e = launch_insert_pass<GDBG_BYTE>(pass, s, n_threads, st, b, hashes, g->hp, g->ts->tp, w); break;
    default: e = launch_insert_pass<GDBG_NIBBLE>(pass, s, n_threads, st, b, hashes, g->hp, g->ts->tp, w); break;
    }
    if (e != cudaSuccess) return fail(GDBG_ERR_CUDA, std::string("insert launch: ") + cudaGetErrorString(e));
    g->launches += 1;
    return GDBG_OK;
}

uint32_t default_bucket_fs(int storage) {
    // 64 KB of table per bucket
    return storage == GDBG_BIT ? 19u : storage == GDBG_NIBBLE ? 17u : 16u;
}

uint32_t default_sort_fs(int storage) {
    // 32 KB of table per bucket (the region and the fresh-cell map fit two
    // CTAs per SM)
    return storage == GDBG_BIT ? 18u : storage == GDBG_NIBBLE ? 16u : 15u;
}

// Can the bucketed path take this batch?  (tables <= 8, every global cell id
// and every record index below 2^32)
bool bucket_fits(const gdbg_graph* g, uint64_t n_kmers, uint32_t fs) {
    const uint64_t n = g->ts->sizes.size();
    if (n > (uint64_t)BK_MAXNT || n_kmers == 0) return false;
    if (n_kmers * n >= (1ull << 32)) return false;
    uint64_t cells = 0;
    for (auto p : g->ts->sizes) cells += ((p + (1ull << fs) - 1) >> fs) << fs;
    return cells <= (1ull << 32);
}

uint64_t buckets_at(const gdbg_graph* g, uint32_t fs) {
    uint64_t nb = 0;
    for (auto p : g->ts->sizes) nb += (p + (1ull << fs) - 1) >> fs;
    return nb;
}

// Bucket size of the segmented path: the set size, else the default 32 KB
// region, made smaller (down to 512 B, within 2^17 buckets) while a bucket of
// the smallest table would get more than 4096 of the batch's records, so a
// bucket's records fit the apply's shared-memory buffer.
uint32_t sort_fs(const gdbg_graph* g, uint64_t n_kmers) {
    if (g->bucket_fs) return g->bucket_fs;
    uint32_t fs = default_sort_fs(g->storage);
    const uint32_t min_fs = g->storage == GDBG_BIT ? 12u : g->storage == GDBG_NIBBLE ? 10u : 9u;
    uint64_t smallest = ~0ull;
    for (auto p : g->ts->sizes) smallest = std::min(smallest, p);
    while (fs > min_fs && (double)n_kmers * (double)(1ull << fs) / (double)smallest > 4096.0 &&
           buckets_at(g, fs - 1) <= (1ull << 17))
        --fs;
    return fs;
}

// Can the segmented bucketed path take this batch?  (bucketed limits at its
// bucket size, at most 2^17 buckets, a shared-memory region of at most 64 KB)
bool sort_fits(const gdbg_graph* g, uint64_t n_kmers) {
    const uint32_t fs = sort_fs(g, n_kmers);
    if (!bucket_fits(g, n_kmers, fs)) return false;
    const uint32_t cpw = g->storage == GDBG_BIT ? 32u : g->storage == GDBG_NIBBLE ? 8u : 4u;
    if (((1ull << fs) / cpw) * 4 > (64u << 10)) return false;
    return buckets_at(g, fs) <= (1ull << 17);
}

enum InsertKind { INS_WINDOWED, INS_PERSISTENT, INS_BUCKETED, INS_SORTED };

// The implementation a batch insert of n_total k-mers takes.
InsertKind insert_kind(const gdbg_graph* g, uint64_t n_total) {
    uint64_t table_bytes = 0;
    for (auto w : g->ts->words) table_bytes += 4 * w;
    const uint32_t fso = g->bucket_fs ? g->bucket_fs : default_bucket_fs(g->storage);
    const bool big = table_bytes >= (256ull << 20) && n_total >= (1ull << 22);
    switch (g->path) {
    case GDBG_PATH_PERSISTENT: return INS_PERSISTENT;
    case GDBG_PATH_BUCKETED_ORDERED:
        return bucket_fits(g, n_total, fso) ? INS_BUCKETED : INS_WINDOWED;
    case GDBG_PATH_BUCKETED:
        if (sort_fits(g, n_total)) return INS_SORTED;
        return bucket_fits(g, n_total, fso) ? INS_BUCKETED : INS_WINDOWED;
    case GDBG_PATH_AUTO:
        if (!big) return INS_WINDOWED;
        if (sort_fits(g, n_total)) return INS_SORTED;
        return bucket_fits(g, n_total, fso) ? INS_BUCKETED : INS_WINDOWED;
    default: return INS_WINDOWED;
    }
}

// Read maps the batch insert will use: the windowed and segmented paths walk
// k-mer runs (tile map), the persistent and ordered bucketed paths warp tasks
// (task map).
int insert_maps(const gdbg_graph* g, uint64_t n_total) {
    if (n_total == UINT64_MAX) return MAP_TILES | MAP_TASKS;
    switch (insert_kind(g, n_total)) {
    case INS_PERSISTENT:
    case INS_BUCKETED: return MAP_TASKS;
    default: return MAP_TILES;
    }
}

int set_error_launch(cudaError_t e, const char* what) {
    return fail(GDBG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Bucketed insert of a read batch: partition the (cell, k-mer) records by
// table region, then apply each region in shared memory.
// counts != nullptr: also the insert_and_query count of every k-mer
// (Byte/Nibble; Bit callers fill ones themselves).
int run_insert_bucketed(gdbg_graph* g, const BatchView& b, uint64_t* n_new, cudaStream_t st,
                        int16_t* counts = nullptr) {
    const uint64_t nk = b.n_kmers, n = g->ts->sizes.size();
    if (nk == 0) {
        if (n_new && b.n_reads) GDBG_CUDA(cudaMemsetAsync(n_new, 0, b.n_reads * sizeof(uint64_t), st));
        return GDBG_OK;
    }
    const uint32_t fs = g->bucket_fs ? g->bucket_fs : default_bucket_fs(g->storage);
    BucketParams bp{};
    bp.fs = fs;
    uint32_t nb = 0;
    for (uint64_t i = 0; i < n; ++i) {
        bp.bbase[i] = nb;
        bp.tbase[i] = (uint64_t)nb << fs;
        bp.twords[i] = (uint32_t)g->ts->words[i];
        nb += (uint32_t)((g->ts->sizes[i] + (1ull << fs) - 1) >> fs);
    }
    bp.bbase[n] = nb;
    bp.n_buckets = nb;
    bp.n_tables = (uint32_t)n;
    bp.total_kmers = b.kofs + b.n_reads;
    const uint64_t nrec = nk * n;
    bp.n_recs = nrec;
    bp.kmer_cap = nk;
    uint32_t bits = 0;
    while ((1ull << bits) < nb) ++bits;
    const uint32_t passes = bits <= 8 ? 1u : (bits + 7) / 8;

    const uint64_t tile_recs = bucket_tile_records();
    const uint64_t tiles = (nrec + tile_recs - 1) / tile_recs;
    const uint64_t hmax = 256 * tiles;
    GDBG_TRY(g->rec_a.ensure(nrec));
    GDBG_TRY(g->rec_b.ensure(nrec));
    GDBG_TRY(g->hist.ensure(hmax));
    GDBG_TRY(g->hist_off.ensure(hmax));
    GDBG_TRY(g->scan_parts.ensure(scan32_partials_needed(hmax) + 1));
    GDBG_TRY(g->bstart.ensure(nb + 1));
    GDBG_TRY(g->new_bits.ensure(nk / 32 + 2));
    GDBG_CUDA(cudaMemsetAsync(g->new_bits.p, 0, (nk / 32 + 2) * sizeof(uint32_t), st));
    GDBG_CUDA(cudaMemsetAsync(g->bstart.p, 0xFF, (nb + 1) * sizeof(uint32_t), st));
    const bool canon = g->shifter == GDBG_CAN_LEMIRE;
    cudaError_t e;
    bp.rout = g->rec_a.p;
    {
        Stage sg(g, "k_bkt_emit", st);
        if ((e = launch_bucket_emit(canon, st, b, g->hp, g->ts->tp, bp)) != cudaSuccess)
            return set_error_launch(e, "bucket emit");
    }
    uint64_t* src = g->rec_a.p;
    uint64_t* dst = g->rec_b.p;
    bp.n_tiles = (uint32_t)tiles;
    bp.hist = g->hist.p;
    bp.offsets = g->hist_off.p;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        bp.shift = 8 * pass;
        bp.rin = src;
        bp.rout = dst;
        {
            Stage sg(g, "k_bkt_hist", st);
            if ((e = launch_bucket_hist((uint32_t)tiles, st, bp)) != cudaSuccess)
                return set_error_launch(e, "bucket histogram");
        }
        {
            Stage sg(g, "k_scan32", st);
            if ((e = launch_scan32(g->hist.p, g->hist_off.p, hmax, g->scan_parts.p, st)) != cudaSuccess)
                return set_error_launch(e, "bucket scan");
        }
        {
            Stage sg(g, "k_bkt_scatter", st);
            if ((e = launch_bucket_scatter(pass + 1 == passes, (uint32_t)tiles, st, bp, g->bstart.p)) != cudaSuccess)
                return set_error_launch(e, "bucket scatter");
        }
        std::swap(src, dst);
        g->launches += 4;   // histogram, 2 scan kernels, scatter
    }
    if ((e = launch_bucket_starts_fix(st, bp, g->bstart.p)) != cudaSuccess)
        return set_error_launch(e, "bucket starts");
    g->launches += 2;
    uint8_t* vals = nullptr;
    if (counts && g->storage != GDBG_BIT) {
        GDBG_TRY(g->iq_vals.ensure(n * nk));
        vals = g->iq_vals.p;
    }
    Stage sg_apply(g, "k_bkt_apply", st);
    if ((e = launch_bucket_apply(g->storage, g->ts->tp, bp, src, g->bstart.p, g->new_bits.p,
                                 g->ts->d_counters, vals, st)) != cudaSuccess)
        return set_error_launch(e, "bucket apply");
    if (vals) {
        if ((e = launch_iq_counts(vals, nk, (uint32_t)n, g->new_bits.p, bp.total_kmers, counts,
                                  false, st)) != cudaSuccess)
            return set_error_launch(e, "insert_and_query counts");
        g->launches += 1;
    }
    if ((e = launch_bucket_read_new(b.kofs, b.n_reads, g->new_bits.p, n_new, g->ts->d_counters, st)) != cudaSuccess)
        return set_error_launch(e, "bucket read counts");
    g->launches += 3;
    return GDBG_OK;
}

// Segmented bucketed insert (gdbg_sort.cuh): emit with first-digit counts,
// one or two unstable digit passes, bucket starts, order-independent apply.
int run_insert_sorted(gdbg_graph* g, const BatchView& b, uint64_t* n_new, cudaStream_t st) {
    const uint64_t nk = b.n_kmers, n = g->ts->sizes.size();
    if (nk == 0) {
        if (n_new && b.n_reads) GDBG_CUDA(cudaMemsetAsync(n_new, 0, b.n_reads * sizeof(uint64_t), st));
        return GDBG_OK;
    }
    const uint32_t fs = sort_fs(g, nk);
    SortParams sp{};
    sp.fs = fs;
    uint32_t nb = 0;
    for (uint64_t i = 0; i < n; ++i) {
        sp.bbase[i] = nb;
        sp.tbase[i] = (uint64_t)nb << fs;
        sp.twords[i] = (uint32_t)g->ts->words[i];
        nb += (uint32_t)((g->ts->sizes[i] + (1ull << fs) - 1) >> fs);
    }
    sp.bbase[n] = nb;
    sp.n_buckets = nb;
    sp.n_tables = (uint32_t)n;
    uint32_t bits = 0;
    while ((1u << bits) < nb) ++bits;
    if (bits <= 8) {
        sp.hi_shift = 0;
        sp.bins1 = 1u << bits;
        sp.bins2 = 1;
    } else {
        sp.hi_shift = bits - 8;
        sp.bins1 = 256;
        sp.bins2 = 1u << sp.hi_shift;
    }
    sp.total_kmers = b.kofs + b.n_reads;
    sp.kmer_cap = nk;
    const uint64_t nrec = nk * n;
    sp.nseg1 = (uint32_t)((nk + SP_SEGK - 1) / SP_SEGK);
    sp.nseg2_cap = sp.bins2 > 1 ? (uint32_t)(nrec / SP_SEG2 + sp.bins1 + 1) : 0u;
    const uint64_t h1 = (uint64_t)sp.bins1 * sp.nseg1;
    const uint64_t h2 = (uint64_t)sp.bins2 * sp.nseg2_cap;
    // reserved pass-2 layout: a bucket of table i gets its expected records
    // (the batch's k-mers times the bucket's share of the table) plus eight
    // standard deviations of a Poisson count; a batch whose k-mers crowd
    // some bucket past that takes the counted layout instead
    uint64_t slots = nrec;
    if (sp.bins2 > 1) {
        uint64_t at = 0;
        for (uint64_t i = 0; i < n; ++i) {
            const double lam = (double)nk * (double)(1ull << fs) / (double)g->ts->sizes[i];
            const uint64_t cap = ((uint64_t)std::ceil(lam + 8.0 * std::sqrt(lam) + 64.0) + 1) & ~1ull;
            sp.cbase[i] = (uint32_t)std::min<uint64_t>(at, 0xFFFFFFFFull);
            sp.bcap[i] = (uint32_t)std::min<uint64_t>(cap, 0xFFFFFFFFull);
            at += (uint64_t)(sp.bbase[i + 1] - sp.bbase[i]) * cap;
        }
        if (at + SP_TILE < 0xFFFFFFFFull && at <= 2 * nrec + (1ull << 20)) {
            slots = at;
        } else {
            for (uint64_t i = 0; i < n; ++i) sp.bcap[i] = sp.cbase[i] = 0;
        }
    }
    sp.n_slots = (uint32_t)slots;
    // reserved pass-1 layout, for the fused emit (four tables, two passes):
    // the device sizes each group from lam[] (k_sp_groups); the same integer
    // sum here gives the slots to allocate
    uint64_t slots1 = nrec;
    bool fused = n == 4 && sp.bins2 > 1 && sp.bins1 == 256;
    if (fused) {
        for (uint64_t i = 0; i < n; ++i)
            sp.lam[i] = ((nk << fs) + g->ts->sizes[i] - 1) / g->ts->sizes[i];
        uint64_t at = 0;
        for (uint32_t grp = 0; grp < 256; ++grp) at += sp_group_cap(sp, grp);
        if (at + 2 * SP_TILE < 0xFFFFFFFFull && at <= 2 * nrec + (1ull << 24)) {
            slots1 = at;
            sp.n_slots1 = (uint32_t)at;
        } else {
            fused = false;
        }
    }
    GDBG_TRY(g->rec_a.ensure(std::max(nrec, slots) + 2));
    GDBG_TRY(g->rec_b.ensure(std::max(nrec, slots1) + 2));
    GDBG_TRY(g->hist.ensure(h1));
    GDBG_TRY(g->hist_off.ensure(h1));
    if (h2) {
        GDBG_TRY(g->sp_hist2.ensure(h2));
        GDBG_TRY(g->sp_off2.ensure(h2));
    }
    GDBG_TRY(g->sp_plan.ensure(4 * (sp.bins1 + 1)));
    if (fused) {
        GDBG_TRY(g->sp_groups.ensure(3 * 256 + 1));
        sp.gcap = g->sp_groups.p;
        sp.gbase = g->sp_groups.p + 256;
        sp.gfill = g->sp_groups.p + 512;
        sp.spill1 = g->sp_groups.p + 768;
    }
    GDBG_TRY(g->scan_parts.ensure(scan32_partials_needed(std::max(h1, h2)) + 1));
    GDBG_TRY(g->bstart.ensure(nb + 1));
    GDBG_TRY(g->sp_end.ensure(nb + 1));
    GDBG_TRY(g->sp_fill.ensure(nb + 1));
    GDBG_TRY(g->new_bits.ensure(nk / 32 + 2));
    sp.spill = g->sp_fill.p;
    sp.bfill = g->sp_fill.p + 1;
    sp.hist1 = g->hist.p;
    sp.off1 = g->hist_off.p;
    sp.hist2 = h2 ? g->sp_hist2.p : nullptr;
    sp.off2 = h2 ? g->sp_off2.p : nullptr;
    sp.plan = g->sp_plan.p;
    sp.err = g->d_err;
    sp.wait_cap = g->copy_polls;
    GDBG_CUDA(cudaMemsetAsync(g->new_bits.p, 0, (nk / 32 + 2) * sizeof(uint32_t), st));
    const bool canon = g->shifter == GDBG_CAN_LEMIRE;
    cudaError_t e;
    // the batch's emit: per copied chunk while a host batch is still
    // arriving (each piece covers the segments whose reads are all in, after
    // its chunk's copy), else one launch
    auto emit = [&](bool fused_kernel, uint64_t* out) -> int {
        auto one = [&](uint32_t s0, uint32_t ns) {
            return fused_kernel ? launch_sp_emit_part(canon, st, b, g->hp, g->ts->tp, sp, out, s0, ns)
                                : launch_sp_emit(canon, st, b, g->hp, g->ts->tp, sp, out, s0, ns);
        };
        if (g->plan.n > 0) {
            uint32_t s0 = 0;
            for (int c = 0; c < g->plan.n; ++c) {
                uint32_t s1 = sp.nseg1;
                if (c + 1 < g->plan.n)
                    s1 = (uint32_t)std::min<uint64_t>(sp.nseg1, g->plan.kmer_end[c] / SP_SEGK);
                if (s1 < s0) s1 = s0;
                GDBG_CUDA(cudaStreamWaitEvent(st, g->chunk_ev[c], 0));
                if (s1 > s0) {
                    if ((e = one(s0, s1 - s0)) != cudaSuccess) return set_error_launch(e, "segment emit");
                    g->launches += 1;
                }
                s0 = s1;
            }
            g->plan.n = 0;
            g->launches -= 1;   // counted by the caller
        } else if ((e = one(0, sp.nseg1)) != cudaSuccess) {
            return set_error_launch(e, "segment emit");
        }
        return GDBG_OK;
    };
    if (fused) {
        // records partitioned as they are made, into the reserved pass-1
        // layout; the separate emit, its counts and the counted pass 1 follow,
        // and work only when a group outgrew its slots
        if ((e = launch_sp_groups(st, sp)) != cudaSuccess) return set_error_launch(e, "segment groups");
        {
            Stage sg(g, "k_sp_emit_part", st);
            GDBG_TRY(emit(true, g->rec_b.p));
        }
        sp.gate1 = sp.spill1;
        {
            Stage sg(g, "k_sp_emit", st);
            GDBG_TRY(emit(false, g->rec_a.p));
        }
        {
            Stage sg(g, "k_scan32", st);
            if ((e = launch_scan32(sp.hist1, sp.off1, h1, g->scan_parts.p, st, sp.gate1)) != cudaSuccess)
                return set_error_launch(e, "segment scan");
        }
        {
            Stage sg(g, "k_sp_part", st);
            if ((e = launch_sp_part(SP_PASS1, st, sp, g->rec_a.p, g->rec_b.p)) != cudaSuccess)
                return set_error_launch(e, "segment partition");
        }
        g->launches += 2;   // groups, fused emit (the rest counted below)
    } else {
        {
            Stage sg(g, "k_sp_emit", st);
            GDBG_TRY(emit(false, g->rec_a.p));
        }
        {
            Stage sg(g, "k_scan32", st);
            if ((e = launch_scan32(sp.hist1, sp.off1, h1, g->scan_parts.p, st)) != cudaSuccess)
                return set_error_launch(e, "segment scan");
        }
        {
            Stage sg(g, "k_sp_part", st);
            if ((e = launch_sp_part(SP_PASS1, st, sp, g->rec_a.p, g->rec_b.p)) != cudaSuccess)
                return set_error_launch(e, "segment partition");
        }
    }
    g->launches += 4;   // emit, 2 scan kernels, partition
    const uint64_t* fin = g->rec_b.p;
    if (sp.bins2 > 1) {
        // the reserved layout first; the counted one (counts, scan, pass)
        // only does work when a bucket outgrew its reserved slots
        const bool reserved = sp.bcap[0] != 0;
        GDBG_CUDA(cudaMemsetAsync(g->sp_fill.p, 0, (nb + 1) * sizeof(uint32_t), st));
        if ((e = launch_sp_plan(st, sp)) != cudaSuccess) return set_error_launch(e, "segment plan");
        if (reserved) {
            Stage sg(g, "k_sp_part", st);
            if ((e = launch_sp_part(SP_PASS2_RESERVED, st, sp, g->rec_b.p, g->rec_a.p)) != cudaSuccess)
                return set_error_launch(e, "segment partition");
        }
        {
            Stage sg(g, "k_sp_hist2", st);
            if ((e = launch_sp_hist2(st, sp, g->rec_b.p)) != cudaSuccess)
                return set_error_launch(e, "segment counts");
        }
        {
            Stage sg(g, "k_scan32", st);
            if ((e = launch_scan32(sp.hist2, sp.off2, h2, g->scan_parts.p, st,
                                   reserved ? sp.spill : nullptr)) != cudaSuccess)
                return set_error_launch(e, "segment scan");
        }
        {
            Stage sg(g, "k_sp_part", st);
            if ((e = launch_sp_part(SP_PASS2_COUNTED, st, sp, g->rec_b.p, g->rec_a.p)) != cudaSuccess)
                return set_error_launch(e, "segment partition");
        }
        fin = g->rec_a.p;
        g->launches += reserved ? 6 : 5;   // plan, [reserved pass], counts, 2 scan kernels, counted pass
    }
    if ((e = launch_sp_starts(st, sp, g->bstart.p, g->sp_end.p)) != cudaSuccess)
        return set_error_launch(e, "bucket starts");
    {
        Stage sg(g, "k_sp_apply", st);
        if ((e = launch_sp_apply(g->storage, g->ts->tp, sp, fin, g->bstart.p, g->sp_end.p, g->new_bits.p,
                                 g->ts->d_counters, st)) != cudaSuccess)
            return set_error_launch(e, "segment apply");
    }
    if ((e = launch_bucket_read_new(b.kofs, b.n_reads, g->new_bits.p, n_new, g->ts->d_counters, st)) != cudaSuccess)
        return set_error_launch(e, "bucket read counts");
    g->launches += 3;   // starts, apply, read counts
    return GDBG_OK;
}

// Persistent cooperative insert of a read batch (one launch per batch).
int run_insert_persistent(gdbg_graph* g, const BatchView& b, uint64_t* n_new, cudaStream_t st) {
    if (b.n_kmers == 0 || b.task_cap == 0) return GDBG_OK;
    const uint64_t W = g->pwindow, n = g->ts->sizes.size();
    GDBG_TRY(g->fresh.ensure(W));
    if (g->storage != GDBG_BIT) GDBG_TRY(g->words_seen.ensure(W * n));
    const uint32_t slots = next_pow2(W * n + W * n / 4);
    if (g->claims.cap < slots) {
        g->claims.release();
        GDBG_TRY(g->claims.ensure(slots));
        GDBG_CUDA(cudaMemsetAsync(g->claims.p, 0, g->claims.cap * sizeof(uint64_t), st));
        g->epoch = 0;
        g->epoch_on_device = false;
    }
    if (!g->epoch_on_device) {
        // hand the host-driven epoch counter to the device
        g->epoch_staging = g->epoch;
        GDBG_CUDA(cudaMemcpyAsync(g->d_epoch, &g->epoch_staging, sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, st));
        g->epoch_on_device = true;
    }
    GDBG_CUDA(cudaMemsetAsync(g->d_bar, 0, 2 * sizeof(unsigned int), st));
    PersistParams pp{};
    pp.spin_cap = g->barrier_polls;
    pp.window_tasks = (uint32_t)(W / TASK_KMERS);
    pp.fresh = g->fresh.p;
    pp.words = g->words_seen.p;
    pp.claims = g->claims.p;
    pp.claims_mask = slots - 1;
    pp.epoch_state = g->d_epoch;
    pp.n_new = (unsigned long long*)n_new;
    pp.counters = g->ts->d_counters;
    pp.err = g->d_err;
    pp.bar = g->d_bar;
    LaunchShape s = g->shape(4);
    int grid = 0;
    cudaError_t e;
    Stage sg(g, "k_insert_persistent", st);
    switch (g->storage) {
    case GDBG_BIT: e = launch_insert_persistent<GDBG_BIT>(s, b.task_cap, st, b, g->hp, g->ts->tp, pp, &grid); break;
    case GDBG_BYTE: e = launch_insert_persistent<GDBG_BYTE>(s, b.task_cap, st, b, g->hp, g->ts->tp, pp, &grid); break;
    default: e = launch_insert_persistent<GDBG_NIBBLE>(s, b.task_cap, st, b, g->hp, g->ts->tp, pp, &grid); break;
    }
    if (e != cudaSuccess)
        return fail(GDBG_ERR_CUDA, std::string("persistent insert launch: ") + cudaGetErrorString(e));
    g->launches += 1;
    return GDBG_OK;
}

// One read's insert in one CTA, its first touchers found in shared memory
// (k_insert_read); done, when given, gets (seq << 32) | the device status
// word as the insert's last write.
int run_insert_read(gdbg_graph* g, const BatchView& b, uint64_t* n_new, uint64_t* done,
                    uint32_t seq, cudaStream_t st) {
    const bool canon = g->shifter == GDBG_CAN_LEMIRE;
    const bool set = !g->read_smem_set;
    cudaError_t e;
    switch (g->storage) {
    case GDBG_BIT:
        e = launch_insert_read<GDBG_BIT>(canon, set, st, b, g->hp, g->ts->tp, n_new, g->ts->d_counters, g->d_err,
                                           done, seq);
        break;
    case GDBG_BYTE:
        e = launch_insert_read<GDBG_BYTE>(canon, set, st, b, g->hp, g->ts->tp, n_new, g->ts->d_counters, g->d_err,
                                           done, seq);
        break;
    default:
        e = launch_insert_read<GDBG_NIBBLE>(canon, set, st, b, g->hp, g->ts->tp, n_new, g->ts->d_counters, g->d_err,
                                           done, seq);
        break;
    }
    if (e != cudaSuccess) return set_error_launch(e, "read insert");
    g->read_smem_set = true;
    g->launches += 1;
    return GDBG_OK;
}

// Windowed probe + commit over n_total k-mers (from the batch or a hash array).
int run_insert(gdbg_graph* g, const BatchView& b, const uint64_t* hashes, uint64_t n_total,
               uint64_t* n_new, cudaStream_t st) {
    if (n_total == 0) return GDBG_OK;
    if (!hashes) {
        // the cooperative kernel only on request: AUTO stays with kernels that
        // never wait on other blocks, so graphs on concurrent streams cannot
        // hold each other's blocks off the GPU
        switch (insert_kind(g, n_total)) {
        case INS_SORTED: return run_insert_sorted(g, b, n_new, st);
        case INS_BUCKETED: return run_insert_bucketed(g, b, n_new, st);
        case INS_PERSISTENT: return run_insert_persistent(g, b, n_new, st);
        default: break;
        }
    }
    if (!hashes && b.n_reads == 1 && g->ts->sizes.size() <= (size_t)READ_INSERT_MAXNT)
        return run_insert_read(g, b, n_new, nullptr, 0, st);   // one read: one CTA
    GDBG_TRY(ensure_insert_scratch(g, st));
    if (g->epoch_on_device) {
        // the device owns the epoch counter: start the host-driven windows
        // from a cleared map
        GDBG_CUDA(cudaMemsetAsync(g->claims.p, 0, g->claims.cap * sizeof(uint64_t), st));
        g->epoch = 0;
        g->epoch_on_device = false;
    }
    const int kpt = hashes ? 4 : (int)g->kpt;
    LaunchShape s = g->shape(kpt);
    for (uint64_t start = 0; start < n_total; start += g->window) {
        uint64_t end = std::min<uint64_t>(n_total, start + g->window);
        GDBG_TRY(next_epoch(g, st));
        WindowParams w;
        w.start = start;
        w.end = end;
        w.fresh = g->fresh.p;
        w.words = g->words_seen.p;
        w.claims = g->claims.p;
        w.claims_mask = g->claims_mask;
        w.epoch = g->epoch;
        w.n_new = (unsigned long long*)n_new;
        w.counters = g->ts->d_counters;
        w.err = g->d_err;
        if (end - start <= (uint64_t)SMALL_BLOCK) {
            // a single read or a small chunk: probe and commit in one block,
            // one k-mer per thread, so no thread updates tables in a chain
            GDBG_TRY(launch_pass(g, 3, s, end - start, st, b, hashes, w));
            continue;
        }
        uint64_t n_threads = (end - start + kpt - 1) / kpt;
        if (n_threads <= (uint64_t)SMALL_BLOCK) {
            // a small window: probe and commit in one block, one launch
            GDBG_TRY(launch_pass(g, 2, s, n_threads, st, b, hashes, w));
            continue;
        }
        GDBG_TRY(launch_pass(g, 0, s, n_threads, st, b, hashes, w));
        GDBG_TRY(launch_pass(g, 1, s, n_threads, st, b, hashes, w));
    }
    return GDBG_OK;
}

// Insert a batch and return every k-mer's insert_and_query count in batch
// order (dbg.hh:327-340 / 249-265 per read).  Needs the bucketed layout,
// where each table region's records are applied in k-mer order.
int run_insert_query(gdbg_graph* g, const BatchView& b, int16_t* counts, uint64_t* n_new,
                     cudaStream_t st) {
    if (b.n_kmers == 0) {
        if (n_new && b.n_reads) GDBG_CUDA(cudaMemsetAsync(n_new, 0, b.n_reads * sizeof(uint64_t), st));
        return GDBG_OK;
    }
    const uint32_t fs = g->bucket_fs ? g->bucket_fs : default_bucket_fs(g->storage);
    if (!bucket_fits(g, b.n_kmers, fs))
        return fail(GDBG_ERR_UNSUPPORTED,
                    "insert_and_query batches need at most 8 tables, 2^32 cells and 2^32 records");
    if (g->storage == GDBG_BIT) {
        GDBG_TRY(run_insert(g, b, nullptr, b.n_kmers, n_new, st));
        cudaError_t e = launch_iq_counts(nullptr, b.n_kmers, 0, nullptr, b.kofs + b.n_reads, counts,
                                         true, st);
        if (e != cudaSuccess) return set_error_launch(e, "insert_and_query counts");
        g->launches += 1;
        return GDBG_OK;
    }
    return run_insert_bucketed(g, b, n_new, st, counts);
}

// Compactor query of a batch (gdbg_compactor.cu): flags and masks per k-mer.
int run_compactor(gdbg_graph* g, const BatchView& b, uint8_t* flags, uint8_t* masks,
                  cudaStream_t st) {
    if (b.n_kmers == 0) return GDBG_OK;
    if (b.n_reads >= 0xFFFFFFFFull) return fail(GDBG_ERR_INVALID_ARG, "too many reads");
    const uint64_t slots = compactor_slots(b.n_kmers, b.n_reads);
    GDBG_TRY(g->cq_keys.ensure(slots));
    GDBG_TRY(g->cq_min.ensure(slots));
    GDBG_TRY(g->cq_ones.ensure(b.n_reads + 1));
    GDBG_CUDA(cudaMemsetAsync(g->cq_keys.p, 0xFF, slots * sizeof(uint64_t), st));
    GDBG_CUDA(cudaMemsetAsync(g->cq_min.p, 0xFF, slots * sizeof(uint32_t), st));
    GDBG_CUDA(cudaMemsetAsync(g->cq_ones.p, 0xFF, (b.n_reads + 1) * sizeof(uint32_t), st));
    cudaError_t e = launch_compactor(g->storage, g->shape(4), st, b, g->hp, g->ts->tp, g->cq_keys.p,
                                     g->cq_min.p, g->cq_ones.p, flags, masks, g->d_err);
    if (e != cudaSuccess) return fail(GDBG_ERR_CUDA, std::string("compactor launch: ") + cudaGetErrorString(e));
    g->launches += 2;
    return GDBG_OK;
}

int run_query(gdbg_graph* g, const BatchView& b, const uint64_t* hashes, uint64_t n_total,
              int16_t* counts, uint64_t* values, cudaStream_t st) {
    if (n_total == 0) return GDBG_OK;
    LaunchShape s = g->shape(4);
    cudaError_t e;
    switch (g->storage) {
    case GDBG_BIT: e = launch_query<GDBG_BIT>(s, n_total, st, b, hashes, g->hp, g->ts->tp, counts, values); break;
    case GDBG_BYTE: e = launch_query<GDBG_BYTE>(s, n_total, st, b, hashes, g->hp, g->ts->tp, counts, values); break;
    default: e = launch_query<GDBG_NIBBLE>(s, n_total, st, b, hashes, g->hp, g->ts->tp, counts, values); break;
    }
    if (e != cudaSuccess) return fail(GDBG_ERR_CUDA, std::string("query launch: ") + cudaGetErrorString(e));
    g->launches += 1;
    return GDBG_OK;
}

int run_masks(gdbg_graph* g, const BatchView& b, uint8_t* masks, cudaStream_t st) {
    if (b.n_kmers == 0) return GDBG_OK;
    LaunchShape s = g->shape(2);
    cudaError_t e;
    switch (g->storage) {
    case GDBG_BIT: e = launch_masks<GDBG_BIT>(s, st, b, g->hp, g->ts->tp, masks); break;
    case GDBG_BYTE: e = launch_masks<GDBG_BYTE>(s, st, b, g->hp, g->ts->tp, masks); break;
    default: e = launch_masks<GDBG_NIBBLE>(s, st, b, g->hp, g->ts->tp, masks); break;
    }
    if (e != cudaSuccess) return fail(GDBG_ERR_CUDA, std::string("mask launch: ") + cudaGetErrorString(e));
    g->launches += 1;
    return GDBG_OK;
}

// Copy a host batch into the handle's staging buffers and prepare it.
// total: the batch's k-mer count when the offsets were built here, else
// UINT64_MAX: the prefix kernel validates the caller's offsets (they must not
// decrease nor run past the packed stream) and computes the total, which
// comes back before anything else is launched.
int stage_host_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                     const uint64_t* offsets, uint64_t n_reads, BatchView* view,
                     bool for_insert = false, uint64_t total = UINT64_MAX) {
    if (!offsets || (n_reads && !packed && n_words))
        return fail(GDBG_ERR_INVALID_ARG, "NULL batch buffers");
    GDBG_TRY(g->st_packed.ensure(n_words + 1));
    GDBG_TRY(g->st_offsets.ensure(n_reads + 1));
    if (n_words)
        GDBG_CUDA(cudaMemcpyAsync(g->st_packed.p, packed, n_words * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(g->st_offsets.p, offsets, (n_reads + 1) * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, g->stream));
    const int maps = for_insert ? (total == UINT64_MAX ? MAP_FOR_INSERT : insert_maps(g, total))
                                : (MAP_TILES | MAP_TASKS);
    return prepare_batch(g, g->st_packed.p, n_words, g->st_offsets.p, n_reads, total, g->stream,
                         view, maps, total == UINT64_MAX);
}

// The handle's second stream for host-to-device copies, with its events.
int ensure_copy_stream(gdbg_graph* g) {
    if (g->copy_stream) return GDBG_OK;
    if (cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        g->copy_stream = nullptr;
        return fail(GDBG_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto& ev : g->chunk_ev)
        GDBG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    GDBG_CUDA(cudaEventCreateWithFlags(&g->prior_ev, cudaEventDisableTiming));
    for (auto& s : g->aslot) {
        GDBG_CUDA(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming));
        GDBG_CUDA(cudaEventCreateWithFlags(&s.released, cudaEventDisableTiming));
    }
    return GDBG_OK;
}

// A host batch for an insert.  The offsets move first and the device prefix
// checks and counts them (with the k-mer prefix at the chunk boundaries); the
// packed reads then move in N_CHUNKS chunks of whole reads, split by bases,
// on copy_stream, and g->plan lets the segmented emit start on each chunk's
// segments as soon as it is in.  Other insert paths wait for the last chunk.
int stage_host_insert(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                      const uint64_t* offsets, uint64_t n_reads, BatchView* view) {
    constexpr int C = gdbg_graph::N_CHUNKS;
    if (!offsets || (n_reads && !packed && n_words))
        return fail(GDBG_ERR_INVALID_ARG, "NULL batch buffers");
    GDBG_TRY(g->st_packed.ensure(n_words + 1));
    GDBG_TRY(g->st_offsets.ensure(n_reads + 1));
    GDBG_TRY(ensure_copy_stream(g));
    // the chunks below wait only for the work the graph's stream holds so far
    // (an earlier batch may still read the staging buffer)
    GDBG_CUDA(cudaEventRecord(g->prior_ev, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(g->st_offsets.p, offsets, (n_reads + 1) * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, g->stream));
    // chunk c holds reads [rb[c], rb[c+1]); the host offsets only choose the
    // split (the device checks them), so any answer here is safe
    uint64_t rb[C + 1];
    rb[0] = 0;
    rb[C] = n_reads;
    const uint64_t b0 = offsets[0], bn = offsets[n_reads];
    for (int c = 1; c < C; ++c) {
        const uint64_t target = bn > b0 ? b0 + (bn - b0) / C * c : b0;
        uint64_t r = (uint64_t)(std::upper_bound(offsets, offsets + n_reads + 1, target) - offsets);
        r = r ? r - 1 : 0;
        rb[c] = std::min(std::max(r, rb[c - 1]), (uint64_t)n_reads);
    }
    // the chunks go out at once and overlap the offsets' copy and check; each
    // chunk's words end at the word of its last base (the word a chunk
    // boundary falls in goes with the earlier chunk, so every chunk's reads
    // are in once its copy and those before it are), all within the packed
    // stream whatever the offsets say
    GDBG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->prior_ev, 0));
    uint64_t w0 = 0;
    for (int c = 0; c < C; ++c) {
        uint64_t w1 = n_words;
        if (c + 1 < C) w1 = std::min<uint64_t>(n_words, (offsets[rb[c + 1]] + 15) / 16);
        if (w1 < w0) w1 = w0;
        if (w1 > w0)
            GDBG_CUDA(cudaMemcpyAsync(g->st_packed.p + w0, packed + w0, (w1 - w0) * sizeof(uint32_t),
                                      cudaMemcpyHostToDevice, g->copy_stream));
        GDBG_CUDA(cudaEventRecord(g->chunk_ev[c], g->copy_stream));
        w0 = w1;
    }
    uint64_t kb[C - 1];
    const int rc = prepare_batch(g, g->st_packed.p, n_words, g->st_offsets.p, n_reads, UINT64_MAX,
                                 g->stream, view, MAP_FOR_INSERT, true, rb + 1, kb, C - 1);
    if (rc != GDBG_OK) {
        cudaStreamSynchronize(g->copy_stream);   // the caller's buffer is read until then
        return rc;
    }
    g->plan.n = C;
    for (int c = 0; c + 1 < C; ++c) g->plan.kmer_end[c] = kb[c];
    return GDBG_OK;
}

// One read of len >= K bases as a batch: offsets {0, len}, k-mer prefix
// {0, n}, task prefix {0, ceil(n / TASK_KMERS)}, zero tile and task maps, a
// zero n_new slot and the packed bases, written into the pinned block and
// copied to the device in one transfer (no prefix or map kernels).
// mapped: the view points at the pinned block itself (no copy); the caller
// synchronises the stream before the block is written again.
int stage_string(gdbg_graph* g, const char* seq, uint64_t len, BatchView* view, bool mapped = false) {
    if (len < g->K) return fail(GDBG_ERR_SEQUENCE_LENGTH, "Sequence must have length >= K");
    if (!seq) return fail(GDBG_ERR_INVALID_ARG, "NULL sequence");
    const uint64_t nk = len - g->K + 1, words = len / 16 + 1;
    const uint64_t tiles = (nk + MAP_TILE - 1) / MAP_TILE;
    const uint64_t tasks = (nk + TASK_KMERS - 1) / TASK_KMERS;
    auto up16 = [](uint64_t x) { return (x + 15) & ~uint64_t(15); };
    const uint64_t o_tile = 64, o_task = up16(o_tile + (tiles + 1) * 4);
    const uint64_t o_pack = up16(o_task + (tasks + 1) * 4), total = o_pack + words * 4;
    // the previous call's copy out of the block has finished
    GDBG_CUDA(cudaEventSynchronize(g->single_done));
    if (g->h_single_cap < total) {
        if (g->h_single) cudaFreeHost(g->h_single);
        g->h_single = nullptr;
        g->h_single_cap = 0;
        const size_t want = std::max<size_t>(total + total / 4, 65536);
        if (cudaHostAlloc((void**)&g->h_single, want, cudaHostAllocMapped) != cudaSuccess) {
            g->h_single = nullptr;
            return fail(GDBG_ERR_OOM, "pinned staging allocation failed");
        }
        void* dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, g->h_single, 0) != cudaSuccess) dp = nullptr;
        g->h_single_dev = static_cast<uint8_t*>(dp);
        g->h_single_cap = want;
    }
    GDBG_TRY(g->d_single.ensure(total));
    uint8_t* h = g->h_single;
    uint32_t* packed = reinterpret_cast<uint32_t*>(h + o_pack);
    std::memset(packed, 0, words * 4);
    for (uint64_t i = 0; i < len; ++i) {
        uint32_t c;
        switch (seq[i]) {
        case 'A': c = 0; break;
        case 'C': c = 1; break;
        case 'G': c = 2; break;
        case 'T': c = 3; break;
        default:
            return fail(GDBG_ERR_INVALID_SEQUENCE,
                        std::string("Alphabet: Invalid symbol '") + seq[i] + "' (alphabet=ACGT)");
        }
        packed[i >> 4] |= c << ((i & 15u) << 1);
    }
    uint64_t* hdr = reinterpret_cast<uint64_t*>(h);
    hdr[0] = 0;        // offsets
    hdr[1] = len;
    hdr[2] = 0;        // k-mer prefix
    hdr[3] = nk;
    hdr[4] = 0;        // task prefix
    hdr[5] = tasks;
    hdr[6] = 0;        // n_new
    hdr[7] = 0;
    std::memset(h + o_tile, 0, o_pack - o_tile);
    uint8_t* d = g->d_single.p;
    if (mapped && g->h_single_dev) {
        d = g->h_single_dev;
    } else {
        GDBG_CUDA(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, g->stream));
        GDBG_CUDA(cudaEventRecord(g->single_done, g->stream));
    }
    view->packed = reinterpret_cast<const uint32_t*>(d + o_pack);
    view->offsets = reinterpret_cast<const uint64_t*>(d);
    view->kofs = reinterpret_cast<const uint64_t*>(d + 16);
    view->tile_read = reinterpret_cast<const uint32_t*>(d + o_tile);
    view->n_reads = 1;
    view->n_kmers = nk;
    view->n_map_tiles = tiles;
    view->tofs = reinterpret_cast<const uint64_t*>(d + 32);
    view->task_read = reinterpret_cast<const uint32_t*>(d + o_task);
    view->task_cap = tasks;
    g->single_nnew = reinterpret_cast<uint64_t*>(d + 48);
    return GDBG_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

const char* gdbg_last_error(void) { return g_last_error.c_str(); }
const char* gdbg_version(void) { return "goetia_gb300 0.1 (sm_103a)"; }

int gdbg_primes_near(uint32_t n, uint64_t x, uint64_t* out, uint32_t* n_out) {
    if (!out || !n_out) return fail(GDBG_ERR_INVALID_ARG, "NULL output");
    uint32_t got = 0;
    if (x == 1) {
        out[0] = 1;
        *n_out = 1;
        return GDBG_OK;
    }
    if (x == 0) {
        *n_out = 0;
        return GDBG_OK;
    }
    auto is_prime = [](uint64_t v) {
        if (v < 2) return false;
        if (v == 2) return true;
        if (v % 2 == 0) return false;
        for (uint64_t i = 3; i * i <= v; i += 2)
            if (v % i == 0) return false;
        return true;
    };
    uint64_t i = x - 1;
    if (i % 2 == 0) i--;
    while (got != n) {
        if (is_prime(i)) out[got++] = i;
        if (i <= 1) break;
        i -= 2;
    }
    *n_out = got;
    return GDBG_OK;
}

int gdbg_create(int storage, int shifter, uint16_t K, uint64_t max_table, uint16_t n_tables,
                gdbg_graph** out) {
    if (n_tables == 0 || n_tables > MAX_TABLES)
        return fail(GDBG_ERR_INVALID_ARG, "n_tables must be in 1..32");
    std::vector<uint64_t> sizes(n_tables);
    uint32_t got = 0;
    GDBG_TRY(gdbg_primes_near(n_tables, max_table, sizes.data(), &got));
    if (got == 0) return fail(GDBG_ERR_INVALID_ARG, "no table sizes below max_table");
    return make_graph(storage, shifter, K, sizes.data(), (uint16_t)got, out);
}

int gdbg_create_sized(int storage, int shifter, uint16_t K, const uint64_t* sizes,
                      uint16_t n_tables, gdbg_graph** out) {
    if (!sizes) return fail(GDBG_ERR_INVALID_ARG, "NULL sizes");
    return make_graph(storage, shifter, K, sizes, n_tables, out);
}

int gdbg_destroy(gdbg_graph* g) {
    if (!g) return GDBG_OK;
    cudaSetDevice(g->device);
    if (g->own_stream) cudaStreamSynchronize(g->own_stream);
    if (g->stream && g->stream != g->own_stream) cudaStreamSynchronize(g->stream);
    g->ts.reset();   // frees the tables with the last handle on them
    if (g->d_err) cudaFree(g->d_err);
    if (g->d_epoch) cudaFree(g->d_epoch);
    if (g->d_bar) cudaFree(g->d_bar);
    if (g->h_single) cudaFreeHost(g->h_single);
    if (g->h_ret) cudaFreeHost(g->h_ret);
    if (g->single_done) cudaEventDestroy(g->single_done);
    if (g->copy_stream) {
        cudaStreamSynchronize(g->copy_stream);
        cudaStreamDestroy(g->copy_stream);
    }
    for (auto& ev : g->chunk_ev)
        if (ev) cudaEventDestroy(ev);
    if (g->prior_ev) cudaEventDestroy(g->prior_ev);
    for (auto& s : g->aslot) {
        if (s.copied) cudaEventDestroy(s.copied);
        if (s.released) cudaEventDestroy(s.released);
        s.packed.release(); s.offsets.release(); s.out.release();
    }
    g->d_single.release();
    g->fresh.release(); g->words_seen.release(); g->claims.release();
    g->kofs.release(); g->tofs.release(); g->partials.release(); g->tile_read.release();
    g->task_read.release();
    g->rec_a.release(); g->rec_b.release(); g->hist.release(); g->hist_off.release();
    g->scan_parts.release(); g->bstart.release(); g->new_bits.release(); g->iq_vals.release();
    g->sp_hist2.release(); g->sp_off2.release(); g->sp_plan.release();
    g->sp_fill.release(); g->sp_end.release();
    g->cq_keys.release(); g->cq_min.release(); g->cq_ones.release();
    g->st_packed.release(); g->st_offsets.release(); g->st_out64.release();
    g->st_out64b.release(); g->st_out64c.release(); g->st_counts.release(); g->st_u8.release();
    for (auto& p : g->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : g->free_events) cudaEventDestroy(e);
    if (g->own_stream) cudaStreamDestroy(g->own_stream);
    delete g;
    return GDBG_OK;
}

int gdbg_clone(const gdbg_graph* g, gdbg_graph** out) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    GDBG_TRY(make_graph(g->storage, g->shifter, g->K, g->ts->sizes.data(), (uint16_t)g->ts->sizes.size(), out));
    (*out)->window = g->window;
    (*out)->kpt = g->kpt;
    (*out)->pwindow = g->pwindow;
    (*out)->persistent = g->persistent;
    (*out)->path = g->path;
    (*out)->bucket_fs = g->bucket_fs;
    return GDBG_OK;
}

int gdbg_share_storage(const gdbg_graph* g, int shifter, uint16_t K, gdbg_graph** out) {
    if (!g || !out) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    GDBG_TRY(check_kinds(g->storage, shifter, K));
    GDBG_TRY(set_device(g));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    gdbg_graph* h = new gdbg_graph();
    h->device = g->device;
    h->ts = g->ts;
    const int rc = init_handle(h, g->storage, shifter, K);
    if (rc != GDBG_OK) {
        gdbg_destroy(h);
        return rc;
    }
    h->window = g->window;
    h->kpt = g->kpt;
    h->pwindow = g->pwindow;
    h->persistent = g->persistent;
    h->path = g->path;
    h->bucket_fs = g->bucket_fs;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        gdbg_destroy(h);
        return fail(GDBG_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = h;
    return GDBG_OK;
}

int gdbg_reset(gdbg_graph* g) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    GDBG_CUDA(cudaMemsetAsync(g->ts->d_tables, 0, g->ts->total_words * sizeof(uint32_t), g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_info(const gdbg_graph* g, int* storage, int* shifter, uint16_t* K, uint16_t* n_tables) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (storage) *storage = g->storage;
    if (shifter) *shifter = g->shifter;
    if (K) *K = g->K;
    if (n_tables) *n_tables = (uint16_t)g->ts->sizes.size();
    return GDBG_OK;
}

int gdbg_get_tablesizes(const gdbg_graph* g, uint64_t* out) {
    if (!g || !out) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    std::copy(g->ts->sizes.begin(), g->ts->sizes.end(), out);
    return GDBG_OK;
}

int gdbg_table_bytes(const gdbg_graph* g, uint64_t* out) {
    if (!g || !out) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    std::copy(g->ts->bytes.begin(), g->ts->bytes.end(), out);
    return GDBG_OK;
}

int gdbg_get_tables(gdbg_graph* g, uint8_t* out, uint64_t out_len) {
    if (!g || !out) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    uint64_t need = 0;
    for (auto b : g->ts->bytes) need += b;
    if (out_len < need) return fail(GDBG_ERR_INVALID_ARG, "output buffer too small");
    GDBG_TRY(set_device(g));
    uint64_t pos = 0;
    for (size_t i = 0; i < g->ts->sizes.size(); ++i) {
        GDBG_CUDA(cudaMemcpyAsync(out + pos, g->ts->d_tables + g->ts->word_off[i], g->ts->bytes[i],
                                  cudaMemcpyDeviceToHost, g->stream));
        pos += g->ts->bytes[i];
    }
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_set_tables(gdbg_graph* g, const uint8_t* in, uint64_t in_len) {
    if (!g || !in) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    uint64_t need = 0;
    for (auto b : g->ts->bytes) need += b;
    if (in_len != need) return fail(GDBG_ERR_INVALID_ARG, "input length does not match the tables");
    GDBG_TRY(set_device(g));
    uint64_t pos = 0;
    for (size_t i = 0; i < g->ts->sizes.size(); ++i) {
        GDBG_CUDA(cudaMemcpyAsync(g->ts->d_tables + g->ts->word_off[i], in + pos, g->ts->bytes[i],
                                  cudaMemcpyHostToDevice, g->stream));
        pos += g->ts->bytes[i];
    }
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_stats(gdbg_graph* g, uint64_t* n_unique, uint64_t* n_occupied) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    unsigned long long c[2];
    GDBG_CUDA(cudaMemcpyAsync(c, g->ts->d_counters, sizeof c, cudaMemcpyDeviceToHost, g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    if (n_unique) *n_unique = c[0];
    if (n_occupied) *n_occupied = c[1];
    return GDBG_OK;
}

// ---- OXLI v4 table files (Storage::save / Storage::load) -------------------
//
// Layout (storage.hh:63-72, bitstorage.cc:151-307, bytestorage.cc:172-290 and
// 480-521, nibblestorage.cc:132-250): "OXLI", version 4, file type (2 Bit,
// 1 Byte, 7 Nibble), [Byte: use_bigcount u8], ksize u32, n_tables u8,
// occupied_bins u64, then per table its size in cells (u64) and its bytes,
// [Byte: bigcount entry count u64 + entries].  Tables move between HBM and
// the file through two pinned staging buffers, so the copy of one chunk
// overlaps the file I/O of the other.

namespace {

constexpr uint8_t OXLI_VERSION = 4;
constexpr uint64_t IO_CHUNK = 32ull << 20;

uint8_t oxli_type(int storage) {
    return storage == GDBG_BIT ? 2 : storage == GDBG_BYTE ? 1 : 7;
}

const char* oxli_noun(int storage) {
    return storage == GDBG_BIT ? "k-mer graph" : "k-mer count";
}

struct FileCloser {
    FILE* f;
    ~FileCloser() { if (f) std::fclose(f); }
};

struct Staging {
    uint8_t* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Staging() {
        for (int i = 0; i < 2; ++i) {
            if (ev[i]) { cudaEventSynchronize(ev[i]); cudaEventDestroy(ev[i]); }
            if (buf[i]) cudaFreeHost(buf[i]);
        }
    }
    int init() {
        for (int i = 0; i < 2; ++i) {
            GDBG_CUDA(cudaHostAlloc((void**)&buf[i], IO_CHUNK, cudaHostAllocDefault));
            GDBG_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        }
        return GDBG_OK;
    }
};

}  // namespace

int gdbg_save(gdbg_graph* g, const char* path) {
    if (!g || !path) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    uint64_t n_occ = 0;
    GDBG_TRY(gdbg_stats(g, nullptr, &n_occ));
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) return fail(GDBG_ERR_IO, std::string("cannot open ") + path + ": " + std::strerror(errno));
    std::vector<uint8_t> head;
    auto put = [&](const void* p, size_t n) {
        head.insert(head.end(), (const uint8_t*)p, (const uint8_t*)p + n);
    };
    const uint8_t ver = OXLI_VERSION, type = oxli_type(g->storage), bigcount = 0;
    const uint32_t ksize = g->K;
    const uint8_t n_tables = (uint8_t)g->ts->sizes.size();
    put("OXLI", 4);
    put(&ver, 1);
    put(&type, 1);
    if (g->storage == GDBG_BYTE) put(&bigcount, 1);
    put(&ksize, 4);
    put(&n_tables, 1);
    put(&n_occ, 8);
    if (std::fwrite(head.data(), 1, head.size(), fc.f) != head.size())
        return fail(GDBG_ERR_IO, std::string("write failed: ") + std::strerror(errno));
    Staging st;
    GDBG_TRY(st.init());
    for (size_t i = 0; i < g->ts->sizes.size(); ++i) {
        const uint64_t size = g->ts->sizes[i], nb = g->ts->bytes[i];
        if (std::fwrite(&size, 8, 1, fc.f) != 1)
            return fail(GDBG_ERR_IO, std::string("write failed: ") + std::strerror(errno));
        const uint8_t* src = (const uint8_t*)(g->ts->d_tables + g->ts->word_off[i]);
        const uint64_t n_chunks = (nb + IO_CHUNK - 1) / IO_CHUNK;
        auto issue = [&](uint64_t c) -> int {
            const uint64_t o = c * IO_CHUNK, len = std::min(IO_CHUNK, nb - o);
            GDBG_CUDA(cudaMemcpyAsync(st.buf[c & 1], src + o, len, cudaMemcpyDeviceToHost, g->stream));
            GDBG_CUDA(cudaEventRecord(st.ev[c & 1], g->stream));
            return GDBG_OK;
        };
        if (n_chunks) GDBG_TRY(issue(0));
        for (uint64_t c = 0; c < n_chunks; ++c) {
            if (c + 1 < n_chunks) GDBG_TRY(issue(c + 1));
            GDBG_CUDA(cudaEventSynchronize(st.ev[c & 1]));
            const uint64_t len = std::min(IO_CHUNK, nb - c * IO_CHUNK);
            if (std::fwrite(st.buf[c & 1], 1, len, fc.f) != len)
                return fail(GDBG_ERR_IO, std::string("write failed: ") + std::strerror(errno));
        }
    }
    if (g->storage == GDBG_BYTE) {
        const uint64_t n_counts = 0;
        if (std::fwrite(&n_counts, 8, 1, fc.f) != 1)
            return fail(GDBG_ERR_IO, std::string("write failed: ") + std::strerror(errno));
    }
    FILE* f = fc.f;
    fc.f = nullptr;
    if (std::fclose(f) != 0)
        return fail(GDBG_ERR_IO, std::string("write failed: ") + std::strerror(errno));
    return GDBG_OK;
}

int gdbg_load(gdbg_graph* g, const char* path, uint16_t* ksize_out) {
    if (!g || !path) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    const std::string file(path), noun(oxli_noun(g->storage));
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return fail(GDBG_ERR_IO, "Cannot open " + noun + " file: " + file);
    const std::string eof_msg = "Unexpected end of " + noun + " file: " + file;
    auto rd = [&](void* p, size_t n) { return std::fread(p, 1, n, fc.f) == n; };
    char sig[4];
    uint8_t ver = 0, type = 0;
    if (!rd(sig, 4) || !rd(&ver, 1) || !rd(&type, 1)) return fail(GDBG_ERR_IO, eof_msg);
    if (std::memcmp(sig, "OXLI", 4) != 0) {
        char hex[16];
        std::string got;
        for (int i = 0; i < 4; ++i) {
            std::snprintf(hex, sizeof hex, "%x", (int)sig[i]);
            got += hex;
        }
        return fail(GDBG_ERR_IO, "Does not start with signature for a oxli file: 0x" + got +
                                     " Should be: OXLI");
    }
    if (ver != OXLI_VERSION)
        return fail(GDBG_ERR_IO, "Incorrect file format version " + std::to_string(ver) +
                                     " while reading " + noun + " file from " + file +
                                     "; should be " + std::to_string(OXLI_VERSION));
    if (type != oxli_type(g->storage))
        return fail(GDBG_ERR_IO, "Incorrect file format type " + std::to_string(type) +
                                     " while reading " + noun + " file from " + file);
    if (g->storage == GDBG_BYTE) {
        uint8_t bigcount = 0;
        if (!rd(&bigcount, 1)) return fail(GDBG_ERR_IO, eof_msg);
        if (bigcount)
            return fail(GDBG_ERR_UNSUPPORTED, "counts above 255 (use_bigcount) are not supported: " + file);
    }
    uint32_t ksize = 0;
    uint8_t n_tables = 0;
    uint64_t n_occ = 0;
    if (!rd(&ksize, 4) || !rd(&n_tables, 1) || !rd(&n_occ, 8)) return fail(GDBG_ERR_IO, eof_msg);
    if (n_tables == 0 || n_tables > MAX_TABLES)
        return fail(GDBG_ERR_UNSUPPORTED, "table count " + std::to_string(n_tables) +
                                              " outside 1.." + std::to_string(MAX_TABLES) + ": " + file);
    // pass 1: table sizes and the file length, before any state changes
    const long data_start = std::ftell(fc.f);
    std::vector<uint64_t> sizes(n_tables);
    for (uint8_t i = 0; i < n_tables; ++i) {
        if (!rd(&sizes[i], 8)) return fail(GDBG_ERR_IO, eof_msg);
        const uint64_t p = sizes[i];
        if (p == 0 || p >= (1ull << 32))
            return fail(GDBG_ERR_UNSUPPORTED, "table size outside 1..2^32-1 cells: " + file);
        const uint64_t nb = g->storage == GDBG_BIT ? p / 8 + 1 : g->storage == GDBG_NIBBLE ? p / 2 + 1 : p;
        if (std::fseek(fc.f, (long)nb, SEEK_CUR) != 0) return fail(GDBG_ERR_IO, eof_msg);
    }
    const long data_end = std::ftell(fc.f);
    if (g->storage == GDBG_BYTE) {
        uint64_t n_counts = 0;
        if (!rd(&n_counts, 8)) return fail(GDBG_ERR_IO, eof_msg);
        if (n_counts)
            return fail(GDBG_ERR_UNSUPPORTED, "bigcount entries are not supported: " + file);
    }
    if (std::fseek(fc.f, 0, SEEK_END) != 0) return fail(GDBG_ERR_IO, eof_msg);
    if (std::ftell(fc.f) < data_end) return fail(GDBG_ERR_IO, eof_msg);
    // new tables (the old ones stay until the new allocation succeeded)
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    if (sizes != g->ts->sizes) {
        std::vector<uint64_t> sz, bytes, words, word_off;
        const uint64_t total = table_layout(g->storage, sizes.data(), n_tables, sz, bytes, words, word_off);
        uint32_t* fresh = nullptr;
        GDBG_CUDA(cudaMalloc((void**)&fresh, total * sizeof(uint32_t)));
        cudaFree(g->ts->d_tables);
        g->ts->d_tables = fresh;
        g->ts->sizes = sz;
        g->ts->bytes = bytes;
        g->ts->words = words;
        g->ts->word_off = word_off;
        g->ts->total_words = total;
        set_table_params(g);
    }
    GDBG_CUDA(cudaMemsetAsync(g->ts->d_tables, 0, g->ts->total_words * sizeof(uint32_t), g->stream));
    // pass 2: table bytes
    if (std::fseek(fc.f, data_start, SEEK_SET) != 0) return fail(GDBG_ERR_IO, eof_msg);
    Staging st;
    GDBG_TRY(st.init());
    uint64_t c_all = 0;  // chunks issued so far, alternating buffers
    for (uint8_t i = 0; i < n_tables; ++i) {
        uint64_t p = 0;
        if (!rd(&p, 8)) return fail(GDBG_ERR_IO, eof_msg);
        uint8_t* dst = (uint8_t*)(g->ts->d_tables + g->ts->word_off[i]);
        const uint64_t nb = g->ts->bytes[i];
        for (uint64_t o = 0; o < nb; o += IO_CHUNK, ++c_all) {
            const uint64_t len = std::min(IO_CHUNK, nb - o);
            const int b = (int)(c_all & 1);
            GDBG_CUDA(cudaEventSynchronize(st.ev[b]));   // its previous copy is done
            if (!rd(st.buf[b], len)) return fail(GDBG_ERR_IO, eof_msg);
            GDBG_CUDA(cudaMemcpyAsync(dst + o, st.buf[b], len, cudaMemcpyHostToDevice, g->stream));
            GDBG_CUDA(cudaEventRecord(st.ev[b], g->stream));
        }
    }
    // occupied bins come from the file; n_unique is kept (bitstorage.cc:264-275)
    unsigned long long occ = n_occ;
    GDBG_CUDA(cudaMemcpyAsync(g->ts->d_counters + 1, &occ, sizeof occ, cudaMemcpyHostToDevice, g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    if (ksize_out) *ksize_out = (uint16_t)ksize;
    return GDBG_OK;
}

int gdbg_update_from(gdbg_graph* g, const gdbg_graph* other) {
    if (!g || !other) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (g->storage != GDBG_BIT || other->storage != GDBG_BIT)
        return fail(GDBG_ERR_UNSUPPORTED, "update_from is defined for BitStorage only");
    if (g->ts->sizes != other->ts->sizes)
        return fail(GDBG_ERR_INVALID_ARG, "both nodegraphs must have same table sizes");
    if (g->device != other->device)
        return fail(GDBG_ERR_INVALID_ARG, "both nodegraphs must be on the same device");
    GDBG_TRY(set_device(g));
    if (g->ts->d_tables == other->ts->d_tables) return GDBG_OK;
    // the merge reads other's tables after all work queued on its stream
    if (other->stream != g->stream) {
        cudaEvent_t ev = nullptr;
        GDBG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t e = cudaEventRecord(ev, other->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g->stream, ev, 0);
        cudaEventDestroy(ev);
        GDBG_CUDA(e);
    }
    GDBG_CUDA(launch_or_merge(g->ts->d_tables, other->ts->d_tables, g->ts->total_words, g->ts->words[0],
                              g->ts->d_counters + 1, g->stream));
    g->launches++;
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_set_stream(gdbg_graph* g, void* stream) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    g->stream = stream ? (cudaStream_t)stream : g->own_stream;
    return GDBG_OK;
}

int gdbg_synchronize(gdbg_graph* g) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return check_device_status(g);
}

// ---- single sequences -------------------------------------------------------

int gdbg_hash(gdbg_graph* g, const char* kmer, uint64_t len, uint64_t* value, uint64_t* fw,
              uint64_t* rc) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (len < g->K)
        return fail(GDBG_ERR_INVALID_SEQUENCE, "HashShifter::hash: Sequence must at least length K");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, kmer, g->K, &b));  // symbols past K are ignored, as in the reference
    GDBG_TRY(g->st_out64.ensure(3));
    GDBG_CUDA(launch_hashes(g->shifter == GDBG_CAN_LEMIRE, g->stream, b, g->hp, g->st_out64.p,
                            g->st_out64.p + 1, g->st_out64.p + 2));
    g->launches += 1;
    uint64_t h[3];
    GDBG_CUDA(cudaMemcpyAsync(h, g->st_out64.p, sizeof h, cudaMemcpyDeviceToHost, g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    if (value) *value = h[0];
    if (fw) *fw = h[1];
    if (rc) *rc = h[2];
    return GDBG_OK;
}

int gdbg_insert_sequence(gdbg_graph* g, const char* seq, uint64_t len, uint64_t* n_kmers,
                         uint64_t* n_new) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    if (g->ts->sizes.size() <= (size_t)READ_INSERT_MAXNT && len >= g->K &&
        insert_kind(g, len - g->K + 1) == INS_WINDOWED) {
        // the read kernel reads the staged block in place and writes the
        // read's count and the device status back into it: no copies, one
        // launch, one synchronisation
        GDBG_TRY(stage_string(g, seq, len, &b, true));
        if (g->h_single_dev) {
            volatile uint64_t* hdr = reinterpret_cast<volatile uint64_t*>(g->h_single);
            uint32_t seq = ++g->read_seq;
            if (seq == 0) seq = g->read_seq = 1;   // 0 is the block's cleared word
            GDBG_TRY(run_insert_read(g, b, g->single_nnew,
                                     reinterpret_cast<uint64_t*>(g->h_single_dev + 56), seq, g->stream));
            // the kernel's last write carries the token: watch for it (up to
            // 2 ms), else wait for the stream, which also reports a failure
            const auto t0 = std::chrono::steady_clock::now();
            bool seen = false;
            for (uint32_t it = 0;; ++it) {
                if ((uint32_t)(hdr[7] >> 32) == seq) {
                    seen = true;
                    break;
                }
                if ((it & 1023u) == 1023u &&
                    std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2))
                    break;
            }
            if (!seen) GDBG_CUDA(cudaStreamSynchronize(g->stream));
            const uint32_t err = (uint32_t)hdr[7];
            if (err) return device_status_fail(g, err);
            if (n_kmers) *n_kmers = len - g->K + 1;
            if (n_new) *n_new = hdr[6];
            return GDBG_OK;
        }
    }
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(run_insert(g, b, nullptr, b.n_kmers, g->single_nnew, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(&g->h_ret->v[0], g->single_nnew, sizeof(uint64_t),
                              cudaMemcpyDeviceToHost, g->stream));
    GDBG_TRY(check_device_status(g));
    if (n_kmers) *n_kmers = len - g->K + 1;
    if (n_new) *n_new = g->h_ret->v[0];
    return GDBG_OK;
}

int gdbg_query_sequence(gdbg_graph* g, const char* seq, uint64_t len, int16_t* counts,
                        uint64_t* hashes) {
    if (!g || !counts) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(g->st_counts.ensure(b.n_kmers));
    if (hashes) GDBG_TRY(g->st_out64.ensure(b.n_kmers));
    GDBG_TRY(run_query(g, b, nullptr, b.n_kmers, g->st_counts.p, hashes ? g->st_out64.p : nullptr,
                       g->stream));
    GDBG_CUDA(cudaMemcpyAsync(counts, g->st_counts.p, b.n_kmers * sizeof(int16_t),
                              cudaMemcpyDeviceToHost, g->stream));
    if (hashes)
        GDBG_CUDA(cudaMemcpyAsync(hashes, g->st_out64.p, b.n_kmers * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_insert_and_query_sequence(gdbg_graph* g, const char* seq, uint64_t len, int16_t* counts,
                                   uint64_t* n_new) {
    if (!g || !counts) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(g->st_counts.ensure(b.n_kmers));
    GDBG_TRY(g->st_out64.ensure(1));
    GDBG_CUDA(cudaMemsetAsync(g->st_out64.p, 0, sizeof(uint64_t), g->stream));
    GDBG_TRY(run_insert_query(g, b, g->st_counts.p, g->st_out64.p, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(counts, g->st_counts.p, b.n_kmers * sizeof(int16_t),
                              cudaMemcpyDeviceToHost, g->stream));
    uint64_t nn = 0;
    GDBG_CUDA(cudaMemcpyAsync(&nn, g->st_out64.p, sizeof nn, cudaMemcpyDeviceToHost, g->stream));
    GDBG_TRY(check_device_status(g));
    if (n_new) *n_new = nn;
    return GDBG_OK;
}

int gdbg_hashes(gdbg_graph* g, const char* seq, uint64_t len, uint64_t* values, uint64_t* fw,
                uint64_t* rc) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(g->st_out64.ensure(b.n_kmers));
    GDBG_TRY(g->st_out64b.ensure(b.n_kmers));
    GDBG_TRY(g->st_out64c.ensure(b.n_kmers));
    GDBG_CUDA(launch_hashes(g->shifter == GDBG_CAN_LEMIRE, g->stream, b, g->hp, g->st_out64.p,
                            g->st_out64b.p, g->st_out64c.p));
    g->launches += 1;
    const size_t nb = b.n_kmers * sizeof(uint64_t);
    if (values) GDBG_CUDA(cudaMemcpyAsync(values, g->st_out64.p, nb, cudaMemcpyDeviceToHost, g->stream));
    if (fw) GDBG_CUDA(cudaMemcpyAsync(fw, g->st_out64b.p, nb, cudaMemcpyDeviceToHost, g->stream));
    if (rc) GDBG_CUDA(cudaMemcpyAsync(rc, g->st_out64c.p, nb, cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_insert_hashes(gdbg_graph* g, const uint64_t* hashes, uint64_t n, uint8_t* is_new) {
    if (!g || (n && !hashes)) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return GDBG_OK;
    if (n >= (1ull << 32)) return fail(GDBG_ERR_INVALID_ARG, "at most 2^32-1 hashes per call");
    GDBG_TRY(set_device(g));
    GDBG_TRY(g->st_out64b.ensure(n));
    GDBG_TRY(g->st_out64.ensure(n));
    GDBG_CUDA(cudaMemcpyAsync(g->st_out64b.p, hashes, n * sizeof(uint64_t), cudaMemcpyHostToDevice,
                              g->stream));
    GDBG_CUDA(cudaMemsetAsync(g->st_out64.p, 0, n * sizeof(uint64_t), g->stream));
    BatchView b{};
    b.n_kmers = n;
    GDBG_TRY(run_insert(g, b, g->st_out64b.p, n, g->st_out64.p, g->stream));
    std::vector<uint64_t> nn(is_new ? n : 0);
    if (is_new)
        GDBG_CUDA(cudaMemcpyAsync(nn.data(), g->st_out64.p, n * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    GDBG_TRY(check_device_status(g));
    for (uint64_t i = 0; is_new && i < n; ++i) is_new[i] = nn[i] ? 1 : 0;
    return GDBG_OK;
}

int gdbg_query_hashes(gdbg_graph* g, const uint64_t* hashes, uint64_t n, int16_t* counts) {
    if (!g || (n && (!hashes || !counts))) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return GDBG_OK;
    GDBG_TRY(set_device(g));
    GDBG_TRY(g->st_out64b.ensure(n));
    GDBG_TRY(g->st_counts.ensure(n));
    GDBG_CUDA(cudaMemcpyAsync(g->st_out64b.p, hashes, n * sizeof(uint64_t), cudaMemcpyHostToDevice,
                              g->stream));
    BatchView b{};
    b.n_kmers = n;
    GDBG_TRY(run_query(g, b, g->st_out64b.p, n, g->st_counts.p, nullptr, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(counts, g->st_counts.p, n * sizeof(int16_t), cudaMemcpyDeviceToHost,
                              g->stream));
    return check_device_status(g);
}

int gdbg_neighbor_masks(gdbg_graph* g, const char* seq, uint64_t len, uint8_t* masks) {
    if (!g || !masks) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(g->st_u8.ensure(b.n_kmers));
    GDBG_TRY(run_masks(g, b, g->st_u8.p, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(masks, g->st_u8.p, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

// ---- packed batches, host buffers ----------------------------------------

int gdbg_insert_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                      const uint64_t* offsets, uint64_t n_reads, uint64_t* n_new,
                      uint64_t* n_kmers) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_insert(g, packed, n_words, offsets, n_reads, &b));
    const cudaEvent_t all_in = g->chunk_ev[gdbg_graph::N_CHUNKS - 1];   // chunks copy in order
    if (insert_kind(g, b.n_kmers) != INS_SORTED) {
        // only the segmented emit starts before the whole batch is in
        GDBG_CUDA(cudaStreamWaitEvent(g->stream, all_in, 0));
        g->plan.n = 0;
    }
    int rc = g->st_out64.ensure(n_reads + 1);
    if (rc == GDBG_OK && n_new && cudaMemsetAsync(g->st_out64.p, 0, n_reads * sizeof(uint64_t),
                                                  g->stream) != cudaSuccess)
        rc = fail(GDBG_ERR_CUDA, "cudaMemsetAsync failed");
    if (rc == GDBG_OK)
        rc = run_insert(g, b, nullptr, b.n_kmers, n_new ? g->st_out64.p : nullptr, g->stream);
    if (g->plan.n) {
        // the plan was not used (an empty batch, or an error before the emit)
        cudaStreamWaitEvent(g->stream, all_in, 0);
        g->plan.n = 0;
    }
    if (rc != GDBG_OK) {
        cudaStreamSynchronize(g->copy_stream);   // the caller's buffer is read until then
        return rc;
    }
    if (n_new && n_reads)
        GDBG_CUDA(cudaMemcpyAsync(n_new, g->st_out64.p, n_reads * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    GDBG_TRY(check_device_status(g));
    if (n_kmers) *n_kmers = b.n_kmers;
    return GDBG_OK;
}

int gdbg_query_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                     const uint64_t* offsets, uint64_t n_reads, int16_t* counts) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_batch(g, packed, n_words, offsets, n_reads, &b));
    if (b.n_kmers && !counts) return fail(GDBG_ERR_INVALID_ARG, "NULL counts");
    GDBG_TRY(g->st_counts.ensure(b.n_kmers + 1));
    GDBG_TRY(run_query(g, b, nullptr, b.n_kmers, g->st_counts.p, nullptr, g->stream));
    if (b.n_kmers)
        GDBG_CUDA(cudaMemcpyAsync(counts, g->st_counts.p, b.n_kmers * sizeof(int16_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_insert_and_query_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                                const uint64_t* offsets, uint64_t n_reads, int16_t* counts,
                                uint64_t* n_new) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_batch(g, packed, n_words, offsets, n_reads, &b));
    if (b.n_kmers && !counts) return fail(GDBG_ERR_INVALID_ARG, "NULL counts");
    GDBG_TRY(g->st_counts.ensure(b.n_kmers + 1));
    GDBG_TRY(g->st_out64.ensure(n_reads + 1));
    if (n_reads) GDBG_CUDA(cudaMemsetAsync(g->st_out64.p, 0, n_reads * sizeof(uint64_t), g->stream));
    GDBG_TRY(run_insert_query(g, b, g->st_counts.p, g->st_out64.p, g->stream));
    if (b.n_kmers)
        GDBG_CUDA(cudaMemcpyAsync(counts, g->st_counts.p, b.n_kmers * sizeof(int16_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    if (n_new && n_reads)
        GDBG_CUDA(cudaMemcpyAsync(n_new, g->st_out64.p, n_reads * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_hashes_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                      const uint64_t* offsets, uint64_t n_reads, uint64_t* values, uint64_t* fw,
                      uint64_t* rc) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_batch(g, packed, n_words, offsets, n_reads, &b));
    const uint64_t n = b.n_kmers + 1;
    GDBG_TRY(g->st_out64.ensure(n));
    GDBG_TRY(g->st_out64b.ensure(n));
    GDBG_TRY(g->st_out64c.ensure(n));
    GDBG_CUDA(launch_hashes(g->shifter == GDBG_CAN_LEMIRE, g->stream, b, g->hp, g->st_out64.p,
                            fw ? g->st_out64b.p : nullptr, rc ? g->st_out64c.p : nullptr));
    g->launches += 1;
    const size_t nb = b.n_kmers * sizeof(uint64_t);
    if (nb && values) GDBG_CUDA(cudaMemcpyAsync(values, g->st_out64.p, nb, cudaMemcpyDeviceToHost, g->stream));
    if (nb && fw) GDBG_CUDA(cudaMemcpyAsync(fw, g->st_out64b.p, nb, cudaMemcpyDeviceToHost, g->stream));
    if (nb && rc) GDBG_CUDA(cudaMemcpyAsync(rc, g->st_out64c.p, nb, cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_neighbor_masks_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                              const uint64_t* offsets, uint64_t n_reads, uint8_t* masks) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_batch(g, packed, n_words, offsets, n_reads, &b));
    if (b.n_kmers && !masks) return fail(GDBG_ERR_INVALID_ARG, "NULL masks");
    GDBG_TRY(g->st_u8.ensure(b.n_kmers + 1));
    GDBG_TRY(run_masks(g, b, g->st_u8.p, g->stream));
    if (b.n_kmers)
        GDBG_CUDA(cudaMemcpyAsync(masks, g->st_u8.p, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

// ---- packed batches, device buffers ---------------------------------------

int gdbg_compactor_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                         const uint64_t* offsets, uint64_t n_reads, uint8_t* flags,
                         uint8_t* masks) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_host_batch(g, packed, n_words, offsets, n_reads, &b));
    if (b.n_kmers && (!flags || !masks)) return fail(GDBG_ERR_INVALID_ARG, "NULL output");
    GDBG_TRY(g->st_u8.ensure(2 * b.n_kmers + 2));
    uint8_t* dflags = g->st_u8.p;
    uint8_t* dmasks = g->st_u8.p + b.n_kmers + 1;
    GDBG_TRY(run_compactor(g, b, dflags, dmasks, g->stream));
    if (b.n_kmers) {
        GDBG_CUDA(cudaMemcpyAsync(flags, dflags, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
        GDBG_CUDA(cudaMemcpyAsync(masks, dmasks, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
    }
    return check_device_status(g);
}

int gdbg_compactor_sequence(gdbg_graph* g, const char* seq, uint64_t len, uint8_t* flags,
                            uint8_t* masks) {
    if (!g || !flags || !masks) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    BatchView b;
    GDBG_TRY(stage_string(g, seq, len, &b));
    GDBG_TRY(g->st_u8.ensure(2 * b.n_kmers + 2));
    uint8_t* dflags = g->st_u8.p;
    uint8_t* dmasks = g->st_u8.p + b.n_kmers + 1;
    GDBG_TRY(run_compactor(g, b, dflags, dmasks, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(flags, dflags, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
    GDBG_CUDA(cudaMemcpyAsync(masks, dmasks, b.n_kmers, cudaMemcpyDeviceToHost, g->stream));
    return check_device_status(g);
}

int gdbg_compactor_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                                const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                                uint8_t* flags, uint8_t* masks, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b));
    if (b.n_kmers && (!flags || !masks)) return fail(GDBG_ERR_INVALID_ARG, "NULL output");
    return run_compactor(g, b, flags, masks, st);
}

int gdbg_insert_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                             const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                             uint64_t* n_new, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b,
                           insert_maps(g, n_kmers_hint)));
    if (n_new && n_reads) GDBG_CUDA(cudaMemsetAsync(n_new, 0, n_reads * sizeof(uint64_t), st));
    return run_insert(g, b, nullptr, b.n_kmers, n_new, st);
}

int gdbg_insert_batch_async(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                            const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers,
                            uint64_t* n_new, void* stream) {
    if (!g || !offsets || (n_words && !packed)) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    if (n_kmers == UINT64_MAX) {
        // counted here from the host offsets (a read whose end lies before
        // its start counts zero, as on the device, which checks them)
        n_kmers = 0;
        for (uint64_t r = 0; r < n_reads; ++r) {
            const uint64_t a = offsets[r], e = offsets[r + 1];
            if (e > a && e - a >= g->K) n_kmers += e - a - g->K + 1;
        }
    }
    if (n_words >= gdbg_graph::ASYNC_SLOT_WORDS) {
        // large batch: its copies go to the next staging slot on copy_stream
        // as soon as the batch two calls back is done with that slot, so they
        // overlap the previous batch's kernels
        GDBG_TRY(ensure_copy_stream(g));
        gdbg_graph::AsyncSlot& s = g->aslot[g->aslot_next];
        if (s.pending && (s.packed.cap < n_words + 1 || s.offsets.cap < n_reads + 1 ||
                          s.out.cap < n_reads + 1))
            GDBG_CUDA(cudaEventSynchronize(s.released));   // regrown below
        GDBG_TRY(s.packed.ensure(n_words + 1));
        GDBG_TRY(s.offsets.ensure(n_reads + 1));
        GDBG_TRY(s.out.ensure(n_reads + 1));
        if (s.pending) GDBG_CUDA(cudaStreamWaitEvent(g->copy_stream, s.released, 0));
        GDBG_CUDA(cudaMemcpyAsync(s.packed.p, packed, n_words * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, g->copy_stream));
        GDBG_CUDA(cudaMemcpyAsync(s.offsets.p, offsets, (n_reads + 1) * sizeof(uint64_t),
                                  cudaMemcpyHostToDevice, g->copy_stream));
        GDBG_CUDA(cudaEventRecord(s.copied, g->copy_stream));
        g->aslot_next ^= 1;
        GDBG_CUDA(cudaStreamWaitEvent(st, s.copied, 0));
        BatchView b;
        int rc = prepare_batch(g, s.packed.p, n_words, s.offsets.p, n_reads, n_kmers, st, &b,
                               insert_maps(g, n_kmers));
        if (rc == GDBG_OK && n_reads &&
            cudaMemsetAsync(s.out.p, 0, n_reads * sizeof(uint64_t), st) != cudaSuccess)
            rc = fail(GDBG_ERR_CUDA, "cudaMemsetAsync failed");
        if (rc == GDBG_OK) rc = run_insert(g, b, nullptr, b.n_kmers, s.out.p, st);
        if (rc == GDBG_OK && n_new && n_reads &&
            cudaMemcpyAsync(n_new, s.out.p, n_reads * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess)
            rc = fail(GDBG_ERR_CUDA, "cudaMemcpyAsync failed");
        // the slot is free again once the work queued on `st` so far is done
        const bool rec = cudaEventRecord(s.released, st) == cudaSuccess;
        s.pending = rec;
        if (rc != GDBG_OK || !rec) {
            cudaStreamSynchronize(g->copy_stream);   // the caller's buffers are read until then
            cudaStreamSynchronize(st);
            s.pending = false;
            return rc != GDBG_OK ? rc : fail(GDBG_ERR_CUDA, "cudaEventRecord failed");
        }
        return GDBG_OK;
    }
    GDBG_TRY(g->st_packed.ensure(n_words + 1));
    GDBG_TRY(g->st_offsets.ensure(n_reads + 1));
    GDBG_TRY(g->st_out64.ensure(n_reads + 1));
    if (n_words)
        GDBG_CUDA(cudaMemcpyAsync(g->st_packed.p, packed, n_words * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, st));
    GDBG_CUDA(cudaMemcpyAsync(g->st_offsets.p, offsets, (n_reads + 1) * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, st));
    BatchView b;
    GDBG_TRY(prepare_batch(g, g->st_packed.p, n_words, g->st_offsets.p, n_reads, n_kmers, st, &b,
                           insert_maps(g, n_kmers)));
    if (n_reads) GDBG_CUDA(cudaMemsetAsync(g->st_out64.p, 0, n_reads * sizeof(uint64_t), st));
    GDBG_TRY(run_insert(g, b, nullptr, b.n_kmers, g->st_out64.p, st));
    if (n_new && n_reads)
        GDBG_CUDA(cudaMemcpyAsync(n_new, g->st_out64.p, n_reads * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, st));
    return GDBG_OK;
}

int gdbg_query_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                            const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                            int16_t* counts, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b));
    return run_query(g, b, nullptr, b.n_kmers, counts, nullptr, st);
}

int gdbg_insert_and_query_batch_device(gdbg_graph* g, const uint32_t* packed,
                                       uint64_t packed_words, const uint64_t* offsets,
                                       uint64_t n_reads, uint64_t n_kmers_hint, int16_t* counts,
                                       uint64_t* n_new, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b));
    if (b.n_kmers && !counts) return fail(GDBG_ERR_INVALID_ARG, "NULL counts");
    if (n_new && n_reads) GDBG_CUDA(cudaMemsetAsync(n_new, 0, n_reads * sizeof(uint64_t), st));
    return run_insert_query(g, b, counts, n_new, st);
}

int gdbg_hashes_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                             const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                             uint64_t* values, uint64_t* fw, uint64_t* rc, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b));
    GDBG_CUDA(launch_hashes(g->shifter == GDBG_CAN_LEMIRE, st, b, g->hp, values, fw, rc));
    g->launches += 1;
    return GDBG_OK;
}

int gdbg_neighbor_masks_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                                     const uint64_t* offsets, uint64_t n_reads,
                                     uint64_t n_kmers_hint, uint8_t* masks, void* stream) {
    if (!g || !offsets) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    cudaStream_t st = pick_stream(g, stream);
    BatchView b;
    GDBG_TRY(prepare_batch(g, packed, packed_words, offsets, n_reads, n_kmers_hint, st, &b));
    return run_masks(g, b, masks, st);
}

// ---- tuning and diagnostics ------------------------------------------------

int gdbg_set_insert_schedule(gdbg_graph* g, uint32_t window_kmers, uint32_t kmers_per_thread) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (window_kmers > (1u << 20))
        return fail(GDBG_ERR_INVALID_ARG, "window must be at most 2^20 k-mers");
    if (kmers_per_thread && kmers_per_thread != 4 && kmers_per_thread != 8)
        return fail(GDBG_ERR_INVALID_ARG, "k-mers per thread must be 4 or 8");
    if (window_kmers) {
        g->window = window_kmers;
        g->pwindow = std::max<uint32_t>(TASK_KMERS, window_kmers / TASK_KMERS * TASK_KMERS);
    }
    if (kmers_per_thread) g->kpt = kmers_per_thread;
    return GDBG_OK;
}

int gdbg_set_insert_path(gdbg_graph* g, int path) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (path < GDBG_PATH_PERSISTENT || path > GDBG_PATH_BUCKETED_ORDERED)
        return fail(GDBG_ERR_INVALID_ARG, "unknown insert path");
    g->path = path;
    return GDBG_OK;
}

int gdbg_set_bucket_bits(gdbg_graph* g, uint32_t log2_cells) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    const uint32_t min_fs = g->storage == GDBG_BIT ? 5u : g->storage == GDBG_NIBBLE ? 3u : 2u;
    if (log2_cells && (log2_cells < min_fs || log2_cells > 20))
        return fail(GDBG_ERR_INVALID_ARG, "bucket size must be 2^k cells, one word <= 2^k <= 2^20");
    if (log2_cells) {
        const uint32_t cpw = g->storage == GDBG_BIT ? 32u : g->storage == GDBG_NIBBLE ? 8u : 4u;
        const uint64_t smem = ((1ull << log2_cells) / cpw) * 4 + 2 * 2 * 2048 * 4 + 1024;
        if (smem > 200 * 1024) return fail(GDBG_ERR_INVALID_ARG, "bucket does not fit shared memory");
    }
    g->bucket_fs = log2_cells;
    return GDBG_OK;
}

int gdbg_set_wait_limits(gdbg_graph* g, uint32_t barrier_polls, uint32_t copy_polls) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    g->barrier_polls = barrier_polls;
    g->copy_polls = copy_polls;
    return GDBG_OK;
}

int gdbg_get_insert_schedule(const gdbg_graph* g, uint32_t* window_kmers, uint32_t* kpt) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    if (window_kmers) *window_kmers = g->window;
    if (kpt) *kpt = g->kpt;
    return GDBG_OK;
}

int gdbg_device_status(gdbg_graph* g, uint32_t* status) {
    if (!g || !status) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    GDBG_CUDA(cudaMemcpyAsync(status, g->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
    GDBG_CUDA(cudaMemsetAsync(g->d_err, 0, sizeof(uint32_t), g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_reserve_staging(gdbg_graph* g, uint64_t max_words, uint64_t max_reads) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    GDBG_TRY(g->st_packed.ensure(max_words + 1));
    GDBG_TRY(g->st_offsets.ensure(max_reads + 1));
    GDBG_TRY(g->st_out64.ensure(max_reads + 1));
    return GDBG_OK;
}

int gdbg_reserve(gdbg_graph* g, uint64_t max_reads, uint64_t max_kmers) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    GDBG_TRY(set_device(g));
    const uint64_t tasks = max_kmers / TASK_KMERS + std::min(max_reads, max_kmers);
    GDBG_TRY(g->kofs.ensure(max_reads + 1));
    GDBG_TRY(g->tofs.ensure(max_reads + 1));
    GDBG_TRY(g->partials.ensure(2 * (max_reads / 1024 + 2)));
    GDBG_TRY(g->tile_read.ensure((max_kmers + MAP_TILE - 1) / MAP_TILE + 1));
    GDBG_TRY(g->task_read.ensure(tasks + 1));
    GDBG_TRY(ensure_insert_scratch(g, g->stream));
    GDBG_CUDA(cudaStreamSynchronize(g->stream));
    return GDBG_OK;
}

int gdbg_set_profiling(gdbg_graph* g, int on) {
    if (!g) return fail(GDBG_ERR_INVALID_ARG, "NULL graph");
    g->profiling = on != 0;
    return GDBG_OK;
}

int gdbg_stage_times(gdbg_graph* g, char* names, uint64_t names_len, double* total_ms,
                     uint64_t* launches, uint32_t max_stages, uint32_t* n_stages) {
    if (!g || !n_stages) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    GDBG_TRY(set_device(g));
    collect_stages(g);
    std::string joined;
    uint32_t n = 0;
    for (auto& acc : g->stage_acc) {
        if (n < max_stages) {
            if (total_ms) total_ms[n] = acc.second.first;
            if (launches) launches[n] = acc.second.second;
        }
        if (!joined.empty()) joined += ",";
        joined += acc.first;
        ++n;
    }
    if (names && names_len) {
        std::strncpy(names, joined.c_str(), names_len - 1);
        names[names_len - 1] = 0;
    }
    *n_stages = n;
    g->stage_acc.clear();
    return GDBG_OK;
}

int gdbg_launch_count(const gdbg_graph* g, uint64_t* launches) {
    if (!g || !launches) return fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    *launches = g->launches;
    return GDBG_OK;
}

}  // extern "C"
