// Batch insert that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host framework that hands out all
// device memory from its own fixed pool and accounts for every byte, or a
// latency-critical loop that must not hit the device-wide synchronisation a
// cudaMalloc / cudaFree implies.  gdbg_insert_batch_noalloc serves them: the
// caller owns the tables, the reads and the outputs (all device memory it got
// its own way), and every scratch buffer the insert needs -- per-read k-mer
// prefix, warp-task map, first-touch claims map, window buffers, barrier and
// counters -- lives in one file-scope static device array of fixed size,
// GDBG_NOALLOC_SCRATCH_BYTES.  Every GPU that loads this library holds that
// array until the process exits.
//
// The array's host-side name is only a stand-in for the device copy, so the
// first call on each device looks its address up with cudaGetSymbolAddress
// (with that device current), zeroes the claims map and the header, and
// remembers the address.  That first call should come before any stream
// capture.  Calls share the array and keep its contents between calls: the
// claims map is epoch-tagged and valid across calls, the counters and the
// barrier are cleared at the start of every call.  Two calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// the array; serialise them.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "gdbg_device.cuh"
#include "gdbg_launch.h"
#include "goetia_gb300.h"

namespace gdbg {
namespace {

constexpr uint64_t NA_MAX_READS = GDBG_NOALLOC_MAX_READS;
constexpr uint64_t NA_MAX_TASKS = GDBG_NOALLOC_MAX_TASKS;
constexpr uint32_t NA_WINDOW = 65536;                  // k-mers per window
constexpr uint32_t NA_SLOTS = 1u << 20;                // >= 1.25 * 8 tables * NA_WINDOW
constexpr uint64_t NA_MAX_TABLES = GDBG_NOALLOC_MAX_TABLES;

constexpr uint64_t align256(uint64_t x) { return (x + 255) / 256 * 256; }

// byte offsets inside the scratch array
constexpr uint64_t OFF_HEADER = 0;                                  // err, bar[2], epoch, counters[2]
constexpr uint64_t OFF_KOFS = 256;
constexpr uint64_t OFF_TOFS = OFF_KOFS + align256((NA_MAX_READS + 1) * 8);
constexpr uint64_t OFF_PARTS = OFF_TOFS + align256((NA_MAX_READS + 1) * 8);
constexpr uint64_t OFF_TASKS = OFF_PARTS + align256(2 * (NA_MAX_READS / 1024 + 2) * 8);
constexpr uint64_t OFF_CLAIMS = OFF_TASKS + align256(NA_MAX_TASKS * 4);
constexpr uint64_t OFF_FRESH = OFF_CLAIMS + align256((uint64_t)NA_SLOTS * 8);
constexpr uint64_t OFF_WORDS = OFF_FRESH + align256((uint64_t)NA_WINDOW * 4);
constexpr uint64_t OFF_END = OFF_WORDS + align256((uint64_t)NA_WINDOW * NA_MAX_TABLES * 4);
static_assert(OFF_END <= GDBG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the static array");

struct Header {
    uint32_t err;
    uint32_t bar[2];
    uint32_t epoch;
    unsigned long long counters[2];
};

}  // namespace
}  // namespace gdbg

static __device__ __align__(256) unsigned char g_noalloc_scratch[GDBG_NOALLOC_SCRATCH_BYTES];

namespace {

int na_fail(int code, const std::string& msg) { return gdbg::report_error(code, msg); }

struct DeviceScratch {
    unsigned char* base = nullptr;
};
std::mutex na_mu;
DeviceScratch na_dev[256];

uint64_t table_bytes(int storage, uint64_t p) {
    return storage == GDBG_BIT ? p / 8 + 1 : storage == GDBG_NIBBLE ? p / 2 + 1 : p;
}

// Once per device, with that device current: the array's device address, and
// the claims map and header cleared.
int setup(int dev, cudaStream_t st, unsigned char** out) {
    std::lock_guard<std::mutex> lk(na_mu);
    if (dev < 0 || dev >= 256) return na_fail(GDBG_ERR_INVALID_ARG, "device ordinal out of range");
    if (!na_dev[dev].base) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return na_fail(GDBG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        unsigned char* base = (unsigned char*)p;
        e = cudaMemsetAsync(base + gdbg::OFF_HEADER, 0, 256, st);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(base + gdbg::OFF_CLAIMS, 0, (size_t)gdbg::NA_SLOTS * 8, st);
        if (e != cudaSuccess)
            return na_fail(GDBG_ERR_CUDA, std::string("scratch clear: ") + cudaGetErrorString(e));
        na_dev[dev].base = base;
    }
    *out = na_dev[dev].base;
    return GDBG_OK;
}

}  // namespace

extern "C" int gdbg_noalloc_table_layout(int storage, const uint64_t* sizes, uint16_t n_tables,
                                         uint64_t* word_offsets) {
    if (!sizes || !word_offsets) return na_fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (storage < GDBG_BIT || storage > GDBG_NIBBLE) return na_fail(GDBG_ERR_INVALID_ARG, "unknown storage kind");
    uint64_t off = 0;
    for (uint16_t i = 0; i < n_tables; ++i) {
        word_offsets[i] = off;
        off += ((table_bytes(storage, sizes[i]) + 3) / 4 + 63) / 64 * 64;
    }
    word_offsets[n_tables] = off;
    return GDBG_OK;
}

extern "C" int gdbg_insert_batch_noalloc(int storage, int shifter, uint16_t K, const uint64_t* sizes,
                                         uint16_t n_tables, uint32_t* tables,
                                         const uint32_t* packed, uint64_t packed_words,
                                         const uint64_t* offsets, uint64_t n_reads,
                                         uint64_t* n_new, uint64_t* stats, void* stream) {
    using namespace gdbg;
    if (storage < GDBG_BIT || storage > GDBG_NIBBLE) return na_fail(GDBG_ERR_INVALID_ARG, "unknown storage kind");
    if (shifter != GDBG_FWD_LEMIRE && shifter != GDBG_CAN_LEMIRE)
        return na_fail(GDBG_ERR_INVALID_ARG, "unknown shifter kind");
    if (K == 0) return na_fail(GDBG_ERR_INVALID_ARG, "K must be positive");
    if (!sizes || !tables || !offsets || (n_reads && !packed))
        return na_fail(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (n_tables == 0 || n_tables > NA_MAX_TABLES)
        return na_fail(GDBG_ERR_INVALID_ARG, "n_tables must be in 1.." + std::to_string(NA_MAX_TABLES));
    for (uint16_t i = 0; i < n_tables; ++i)
        if (sizes[i] == 0 || sizes[i] >= (1ull << 32))
            return na_fail(GDBG_ERR_INVALID_ARG, "table sizes must be in 1..2^32-1 cells");
    if (n_reads > NA_MAX_READS)
        return na_fail(GDBG_ERR_INVALID_ARG, "n_reads exceeds the no-alloc maximum of " +
                                                 std::to_string(NA_MAX_READS));
    // every read adds at most one partial warp task; the stream bounds the k-mers
    const uint64_t task_bound = packed_words / 2 + n_reads;
    if (task_bound > NA_MAX_TASKS)
        return na_fail(GDBG_ERR_INVALID_ARG,
                       "batch too large for the no-alloc scratch: packed_words/2 + n_reads must be <= " +
                           std::to_string(NA_MAX_TASKS));
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(GDBG_ERR_CUDA, cudaGetErrorString(e));
    unsigned char* base = nullptr;
    int rc = setup(dev, st, &base);
    if (rc != GDBG_OK) return rc;

    Header* hdr = (Header*)(base + OFF_HEADER);
    uint64_t* kofs = (uint64_t*)(base + OFF_KOFS);
    uint64_t* tofs = (uint64_t*)(base + OFF_TOFS);
    uint64_t* parts = (uint64_t*)(base + OFF_PARTS);
    uint32_t* task_read = (uint32_t*)(base + OFF_TASKS);
    // clear what must start at zero: status, barrier, counters (not the epoch)
    if ((e = cudaMemsetAsync(hdr, 0, offsetof(Header, epoch), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(&hdr->counters, 0, sizeof hdr->counters, st)) != cudaSuccess ||
        (n_new && n_reads && (e = cudaMemsetAsync(n_new, 0, n_reads * 8, st)) != cudaSuccess))
        return na_fail(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (n_reads) {
        int nl = 0;
        if ((e = launch_kmer_prefix(offsets, n_reads, K, packed_words * 16, parts, kofs, tofs,
                                    &hdr->err, st, &nl)) != cudaSuccess ||
            (e = launch_task_map(tofs, n_reads, NA_MAX_TASKS, task_read, st)) != cudaSuccess)
            return na_fail(GDBG_ERR_CUDA, std::string("batch preparation: ") + cudaGetErrorString(e));

        TableParams tp{};
        uint64_t off = 0;
        for (uint16_t i = 0; i < n_tables; ++i) {
            tp.words[i] = tables + off;
            tp.p[i] = sizes[i];
            tp.m[i] = ~0ull / sizes[i];
            off += ((table_bytes(storage, sizes[i]) + 3) / 4 + 63) / 64 * 64;
        }
        tp.n = n_tables;
        const HashParams hp = make_hash_params(K);
        BatchView b{};
        b.packed = packed;
        b.offsets = offsets;
        b.kofs = kofs;
        b.tofs = tofs;
        b.task_read = task_read;
        b.task_cap = task_bound;
        b.n_reads = n_reads;
        b.n_kmers = UINT64_MAX;
        PersistParams pp{};
        pp.window_tasks = NA_WINDOW / TASK_KMERS;
        pp.fresh = (uint32_t*)(base + OFF_FRESH);
        pp.words = (uint32_t*)(base + OFF_WORDS);
        pp.claims = (uint64_t*)(base + OFF_CLAIMS);
        pp.claims_mask = NA_SLOTS - 1;
        pp.epoch_state = &hdr->epoch;
        pp.n_new = (unsigned long long*)n_new;
        pp.counters = hdr->counters;
        pp.err = &hdr->err;
        pp.bar = hdr->bar;
        LaunchShape s{shifter == GDBG_CAN_LEMIRE, 4, (int)n_tables};
        int grid = 0;
        switch (storage) {
        case GDBG_BIT: e = launch_insert_persistent<GDBG_BIT>(s, task_bound, st, b, hp, tp, pp, &grid); break;
        case GDBG_BYTE: e = launch_insert_persistent<GDBG_BYTE>(s, task_bound, st, b, hp, tp, pp, &grid); break;
        default: e = launch_insert_persistent<GDBG_NIBBLE>(s, task_bound, st, b, hp, tp, pp, &grid); break;
        }
        if (e != cudaSuccess) return na_fail(GDBG_ERR_CUDA, std::string("insert launch: ") + cudaGetErrorString(e));
    }
    if (stats) {
        if ((e = cudaMemcpyAsync(stats, hdr->counters, 16, cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(stats + 2, 0, 8, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(stats + 2, &hdr->err, 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
            return na_fail(GDBG_ERR_CUDA, cudaGetErrorString(e));
        return GDBG_OK;
    }
    // no stats buffer to carry the device status: wait for the insert and
    // report a failed device-side check here, before the next call clears it
    uint32_t err = 0;
    if ((e = cudaMemcpyAsync(&err, &hdr->err, sizeof err, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return na_fail(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (err)
        return na_fail(GDBG_ERR_DEVICE,
                       "device status 0x" + [&] {
                           char b[16];
                           std::snprintf(b, sizeof b, "%x", err);
                           return std::string(b);
                       }() + " (1=CAS cap, 2=claims map full, 4=barrier timeout, 8=bad read offsets)");
    return GDBG_OK;
}
