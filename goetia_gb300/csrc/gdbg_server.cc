// Serving runtime: many sample streams, each with its own dBG resident in
// HBM, fed with read chunks as they are released (gdbg_server_* in
// include/goetia_gb300.h).
//
// The reference's streaming driver (goetia/processors.py:39-498,
// AsyncSequenceProcessor over processors.hh:304-331) consumes one sample at a
// time in one worker thread.  Here one process serves many samples at once on
// one GPU, with the request loop in native threads:
//
//   * admission thread: a stream is admitted -- its graph created, its
//     tables, insert scratch and staging allocated -- when its first chunk is
//     due (or due within the look-ahead and nothing else waits) and its
//     footprint fits the HBM budget; streams are admitted in the order their
//     first chunks are due, so a large stream waiting for room holds back the
//     ones behind it.  A drained stream returns its budget share at once but
//     its device memory is freed lazily, only when an admission needs the
//     room (freeing device memory waits for the whole device).
//   * dispatcher threads (streams dealt round-robin over them): each chunk is
//     copied into one of its stream's pinned staging slots and handed to
//     gdbg_insert_batch_async on the stream's own CUDA stream, up to `depth`
//     chunks of a stream in flight, so chunks of different streams overlap on
//     the device while each stream's chunks apply in release order; an event
//     after each chunk is polled, and on completion the per-read new counts
//     are copied to the caller and the latency (completion - release) logged.
//
// Every graph is used by one dispatcher thread only after the admission
// thread has built it, as the C ABI requires (calls on one handle
// serialised).  Per-chunk results equal a sequential replay of each stream.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "gdbg_launch.h"
#include "goetia_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

int sfail(int code, const std::string& msg) { return gdbg::report_error(code, msg); }

uint64_t table_bytes_of(int storage, uint64_t p) {
    return storage == GDBG_BIT ? p / 8 + 1 : storage == GDBG_NIBBLE ? p / 2 + 1 : p;
}

struct Chunk {
    const uint32_t* packed;
    uint64_t n_words;
    const uint64_t* offsets;
    uint64_t n_reads, n_kmers;
    double release;
    uint64_t* n_new;
    uint64_t tag;
};

struct Slot {
    uint32_t* h_packed = nullptr;
    uint64_t* h_off = nullptr;
    uint64_t* h_new = nullptr;
    cudaEvent_t ev = nullptr;
    Chunk c{};
};

enum StreamState { S_WAITING, S_ACTIVE, S_DRAINED, S_FREED };

struct SStream {
    uint64_t id = 0, max_table = 0, max_reads = 0, max_words = 0, footprint = 0;
    std::mutex mu;                 // guards queue, finished, submitted
    std::deque<Chunk> queue;       // submitted, not yet dispatched
    bool finished = false;
    uint64_t submitted = 0;
    std::atomic<int> state{S_WAITING};
    gdbg_graph* g = nullptr;
    cudaStream_t cs = nullptr;     // the stream's own CUDA stream (the graph runs on it)
    std::vector<Slot> slots;
    std::vector<int> free_slots;
    std::deque<int> inflight;
    uint64_t done = 0;
    uint32_t device_status = 0;
    bool waited = false;           // its first chunk came due while it did not fit
};

struct Completion {
    uint64_t tag;
    double latency, done;
    int ok;
};

}  // namespace

struct gdbg_server {
    int storage = 0, shifter = 0, device = 0;
    uint16_t K = 0, n_tables = 0;
    uint64_t budget = 0;
    uint32_t depth = 2, n_dispatch = 1;
    uint32_t window = 262144;
    double lookahead = 0.05;

    std::vector<std::unique_ptr<SStream>> streams;   // in declaration order
    std::unordered_map<uint64_t, SStream*> by_id;

    std::atomic<bool> started{false}, stop{false};
    Clock::time_point t0;
    std::thread admitter;
    std::vector<std::thread> dispatchers;

    // streams handed to each dispatcher (append-only, guarded by hand_mu)
    std::mutex hand_mu;
    std::vector<std::vector<SStream*>> handed;
    std::atomic<uint64_t> hand_version{0};

    std::mutex budget_mu;
    uint64_t used = 0, peak = 0, zombie_bytes = 0;
    std::vector<SStream*> zombies;

    std::mutex done_mu;
    std::vector<Completion> completions;
    size_t polled = 0;

    std::atomic<uint64_t> submitted{0}, finished_chunks{0}, failed{0}, kmers{0};
    std::atomic<uint64_t> admitted{0}, admission_waits{0}, lazy_frees{0};
    std::atomic<uint32_t> device_status{0};
    std::mutex stat_mu;
    double first_dispatch = -1, last_done = -1;
    double admit_max = 0, admit_total = 0, dispatch_max = 0, dispatch_total = 0;
    std::string last_error;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes of a stream: tables, the windowed insert's scratch, the
// host-call staging of its largest chunk and the batch maps.
uint64_t footprint(const gdbg_server* s, uint64_t max_table, uint64_t max_reads, uint64_t max_words) {
    std::vector<uint64_t> p(s->n_tables);
    uint32_t got = 0;
    if (gdbg_primes_near(s->n_tables, max_table, p.data(), &got) != GDBG_OK) got = 0;
    uint64_t tables = 0;
    for (uint32_t i = 0; i < got; ++i) tables += (table_bytes_of(s->storage, p[i]) + 255) / 256 * 256;
    uint64_t slots = 1;
    while (slots < 2ull * s->window * s->n_tables) slots <<= 1;
    const uint64_t scratch = slots * 8 * 5 / 4 + (uint64_t)s->window * 4 * (1 + s->n_tables);
    const uint64_t staging = (max_words + 1) * 4 + (2 * max_reads + 2) * 8 * 5 / 4;
    const uint64_t maps = (max_reads + 1) * 16 + (max_words * 16 / 1024 + 2) * 4;
    return tables + scratch + staging + maps;
}

void free_stream_memory(SStream* st) {
    if (st->g) gdbg_destroy(st->g);   // waits for the stream's work
    st->g = nullptr;
    if (st->cs) cudaStreamDestroy(st->cs);
    st->cs = nullptr;
    for (auto& sl : st->slots) {
        if (sl.h_packed) cudaFreeHost(sl.h_packed);
        if (sl.h_off) cudaFreeHost(sl.h_off);
        if (sl.h_new) cudaFreeHost(sl.h_new);
        if (sl.ev) cudaEventDestroy(sl.ev);
    }
    st->slots.clear();
    st->state.store(S_FREED);
}

// Graph, slots and events of an admitted stream.
int build_stream(gdbg_server* s, SStream* st) {
    int rc = gdbg_create(s->storage, s->shifter, s->K, st->max_table, s->n_tables, &st->g);
    if (rc == GDBG_OK && cudaStreamCreateWithFlags(&st->cs, cudaStreamNonBlocking) != cudaSuccess)
        rc = sfail(GDBG_ERR_CUDA, "serving: stream creation failed");
    if (rc == GDBG_OK) rc = gdbg_set_stream(st->g, st->cs);
    if (rc == GDBG_OK) rc = gdbg_set_insert_path(st->g, GDBG_PATH_WINDOWED);
    if (rc == GDBG_OK) rc = gdbg_set_insert_schedule(st->g, s->window, 4);
    const uint64_t max_kmers = st->max_words * 16;
    if (rc == GDBG_OK) rc = gdbg_reserve(st->g, st->max_reads, max_kmers);
    if (rc == GDBG_OK) rc = gdbg_reserve_staging(st->g, st->max_words, st->max_reads);
    if (rc != GDBG_OK) return rc;
    st->slots.resize(s->depth);
    for (uint32_t i = 0; i < s->depth; ++i) {
        Slot& sl = st->slots[i];
        if (cudaHostAlloc((void**)&sl.h_packed, (st->max_words + 1) * 4, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.h_off, (st->max_reads + 1) * 8, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.h_new, (st->max_reads + 1) * 8, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess)
            return sfail(GDBG_ERR_OOM, "serving: pinned staging allocation failed");
        st->free_slots.push_back((int)i);
    }
    return GDBG_OK;
}

void record_error(gdbg_server* s, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->stat_mu);
    s->last_error = msg;
}

// Release time of a stream's next chunk, or a negative value when it has none
// queued (and whether it will get none).
double head_release(SStream* st, bool* none_left) {
    std::lock_guard<std::mutex> lk(st->mu);
    *none_left = st->queue.empty() && st->finished;
    return st->queue.empty() ? -1.0 : st->queue.front().release;
}

void admission_loop(gdbg_server* s) {
    cudaSetDevice(s->device);
    uint32_t rr = 0;
    size_t left = s->streams.size();
    while (!s->stop.load() && left) {
        // the waiting stream whose next chunk is due first (declaration order
        // breaks ties); streams without chunks yet do not hold others back
        SStream* st = nullptr;
        double rel = 0;
        for (auto& p : s->streams) {
            if (p->state.load() != S_WAITING) continue;
            bool none_left = false;
            const double r = head_release(p.get(), &none_left);
            if (none_left) {   // finished without chunks: nothing to admit
                p->state.store(S_DRAINED);
                --left;
                continue;
            }
            if (r >= 0 && (!st || r < rel)) {
                st = p.get();
                rel = r;
            }
        }
        const double now = s->now();
        if (!st || rel > now + s->lookahead) {
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            continue;
        }
        {
            std::unique_lock<std::mutex> lk(s->budget_mu);
            if (s->used + s->zombie_bytes + st->footprint > s->budget && !s->zombies.empty()) {
                // drained streams still hold device memory: free it now
                std::vector<SStream*> z;
                z.swap(s->zombies);
                s->zombie_bytes = 0;
                lk.unlock();
                for (SStream* x : z) free_stream_memory(x);
                s->lazy_frees.fetch_add(1);
                continue;
            }
            if (s->used + st->footprint > s->budget) {
                lk.unlock();
                if (rel <= now && !st->waited) {
                    st->waited = true;
                    s->admission_waits.fetch_add(1);
                }
                std::this_thread::sleep_for(std::chrono::microseconds(50));
                continue;
            }
            s->used += st->footprint;
            s->peak = std::max(s->peak, s->used + s->zombie_bytes);
        }
        const double a0 = s->now();
        const int rc = build_stream(s, st);
        const double a1 = s->now();
        {
            std::lock_guard<std::mutex> lk(s->stat_mu);
            s->admit_max = std::max(s->admit_max, a1 - a0);
            s->admit_total += a1 - a0;
        }
        --left;
        if (rc != GDBG_OK) {
            record_error(s, std::string("admission: ") + gdbg_last_error());
            // its chunks fail; the budget share goes back
            {
                std::lock_guard<std::mutex> lk(st->mu);
                for (const Chunk& c : st->queue) {
                    std::lock_guard<std::mutex> ld(s->done_mu);
                    s->completions.push_back({c.tag, -1.0, a1, 0});
                }
                s->failed.fetch_add(st->queue.size());
                s->finished_chunks.fetch_add(st->queue.size());
                st->queue.clear();
                st->finished = true;
            }
            std::lock_guard<std::mutex> lb(s->budget_mu);
            s->used -= st->footprint;
            st->state.store(S_DRAINED);
            continue;
        }
        s->admitted.fetch_add(1);
        st->state.store(S_ACTIVE);
        {
            std::lock_guard<std::mutex> lk(s->hand_mu);
            s->handed[rr % s->n_dispatch].push_back(st);
            ++rr;
        }
        s->hand_version.fetch_add(1);
    }
}

// Complete and dispatch on one stream; true when it did any work.
bool serve_stream(gdbg_server* s, SStream* st) {
    bool work = false;
    // completions, in order
    while (!st->inflight.empty()) {
        Slot& sl = st->slots[st->inflight.front()];
        const cudaError_t q = cudaEventQuery(sl.ev);
        if (q == cudaErrorNotReady) break;
        const double t = s->now();
        const int ok = q == cudaSuccess;
        if (ok && sl.c.n_new && sl.c.n_reads) std::memcpy(sl.c.n_new, sl.h_new, sl.c.n_reads * 8);
        if (!ok) {
            s->failed.fetch_add(1);
            record_error(s, std::string("serving: chunk failed: ") + cudaGetErrorString(q));
        }
        {
            std::lock_guard<std::mutex> lk(s->done_mu);
            s->completions.push_back({sl.c.tag, t - sl.c.release, t, ok});
        }
        {
            std::lock_guard<std::mutex> lk(s->stat_mu);
            s->last_done = std::max(s->last_done, t);
        }
        s->kmers.fetch_add(sl.c.n_kmers);
        s->finished_chunks.fetch_add(1);
        st->free_slots.push_back(st->inflight.front());
        st->inflight.pop_front();
        ++st->done;
        work = true;
    }
    // dispatch released chunks while a slot is free
    while (!st->free_slots.empty()) {
        Chunk c;
        {
            std::lock_guard<std::mutex> lk(st->mu);
            if (st->queue.empty() || st->queue.front().release > s->now()) break;
            c = st->queue.front();
            st->queue.pop_front();
        }
        const double d0 = s->now();
        const int si = st->free_slots.back();
        st->free_slots.pop_back();
        Slot& sl = st->slots[si];
        sl.c = c;
        if (c.n_words) std::memcpy(sl.h_packed, c.packed, c.n_words * 4);
        std::memcpy(sl.h_off, c.offsets, (c.n_reads + 1) * 8);
        int rc = gdbg_insert_batch_async(st->g, sl.h_packed, c.n_words, sl.h_off, c.n_reads,
                                         c.n_kmers, sl.h_new, nullptr);
        if (rc == GDBG_OK && cudaEventRecord(sl.ev, st->cs) != cudaSuccess)
            rc = sfail(GDBG_ERR_CUDA, "serving: cudaEventRecord failed");
        const double d1 = s->now();
        {
            std::lock_guard<std::mutex> lk(s->stat_mu);
            if (s->first_dispatch < 0) s->first_dispatch = d0;
            s->dispatch_max = std::max(s->dispatch_max, d1 - d0);
            s->dispatch_total += d1 - d0;
        }
        if (rc != GDBG_OK) {
            record_error(s, std::string("serving: dispatch failed: ") + gdbg_last_error());
            s->failed.fetch_add(1);
            s->finished_chunks.fetch_add(1);
            std::lock_guard<std::mutex> lk(s->done_mu);
            s->completions.push_back({c.tag, -1.0, d1, 0});
            st->free_slots.push_back(si);
            continue;
        }
        st->inflight.push_back(si);
        work = true;
    }
    return work;
}

}  // namespace

namespace {

// Drained: no chunk queued or in flight and no more to come.
bool drained(SStream* st) {
    if (!st->inflight.empty()) return false;
    std::lock_guard<std::mutex> lk(st->mu);
    return st->finished && st->queue.empty();
}

void dispatch_loop(gdbg_server* s, uint32_t me) {
    cudaSetDevice(s->device);
    std::vector<SStream*> mine;
    uint64_t seen = ~0ull;
    for (;;) {
        const uint64_t v = s->hand_version.load();
        if (v != seen) {
            std::lock_guard<std::mutex> lk(s->hand_mu);
            for (size_t i = mine.size(); i < s->handed[me].size(); ++i) mine.push_back(s->handed[me][i]);
            seen = v;
        }
        bool work = false;
        for (SStream* st : mine) {
            if (st->state.load() != S_ACTIVE) continue;
            work |= serve_stream(s, st);
            if (drained(st)) {
                // device-side checks of the stream's inserts, then its budget
                // share goes back (its memory is freed lazily)
                uint32_t status = 0;
                if (gdbg_device_status(st->g, &status) == GDBG_OK && status) {
                    st->device_status |= status;
                    s->device_status.fetch_or(status);
                }
                st->state.store(S_DRAINED);
                std::lock_guard<std::mutex> lk(s->budget_mu);
                s->used -= st->footprint;
                s->zombies.push_back(st);
                s->zombie_bytes += st->footprint;
                work = true;
            }
        }
        if (s->stop.load()) {
            bool all_done = true;
            for (SStream* st : mine) all_done &= st->state.load() != S_ACTIVE;
            if (all_done) return;
        }
        if (!work) std::this_thread::yield();
    }
}

}  // namespace

extern "C" {

int gdbg_server_create(int storage, int shifter, uint16_t K, uint16_t n_tables,
                       uint64_t hbm_budget, uint32_t depth, uint32_t dispatch_threads,
                       gdbg_server** out) {
    if (!out) return sfail(GDBG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (storage < GDBG_BIT || storage > GDBG_NIBBLE) return sfail(GDBG_ERR_INVALID_ARG, "unknown storage kind");
    if (shifter != GDBG_FWD_LEMIRE && shifter != GDBG_CAN_LEMIRE)
        return sfail(GDBG_ERR_INVALID_ARG, "unknown shifter kind");
    if (K == 0 || n_tables == 0 || depth == 0 || depth > 64 || dispatch_threads == 0 ||
        dispatch_threads > 64)
        return sfail(GDBG_ERR_INVALID_ARG, "K, n_tables, depth (1..64) and dispatch threads (1..64) must be positive");
    auto* s = new gdbg_server();
    s->storage = storage;
    s->shifter = shifter;
    s->K = K;
    s->n_tables = n_tables;
    s->budget = hbm_budget;
    s->depth = depth;
    s->n_dispatch = dispatch_threads;
    s->handed.resize(dispatch_threads);
    cudaGetDevice(&s->device);
    *out = s;
    return GDBG_OK;
}

int gdbg_server_stream(gdbg_server* s, uint64_t stream_id, uint64_t max_table,
                       uint64_t max_chunk_reads, uint64_t max_chunk_words) {
    if (!s) return sfail(GDBG_ERR_INVALID_ARG, "NULL server");
    if (s->started.load()) return sfail(GDBG_ERR_INVALID_ARG, "streams are declared before gdbg_server_start");
    if (s->by_id.count(stream_id)) return sfail(GDBG_ERR_INVALID_ARG, "stream declared twice");
    if (max_table < 2) return sfail(GDBG_ERR_INVALID_ARG, "max_table must be at least 2");
    auto st = std::make_unique<SStream>();
    st->id = stream_id;
    st->max_table = max_table;
    st->max_reads = std::max<uint64_t>(max_chunk_reads, 1);
    st->max_words = std::max<uint64_t>(max_chunk_words, 1);
    st->footprint = footprint(s, max_table, st->max_reads, st->max_words);
    if (st->footprint > s->budget)
        return sfail(GDBG_ERR_OOM, "stream " + std::to_string(stream_id) + " needs " +
                                       std::to_string(st->footprint) + " bytes, over the HBM budget");
    s->by_id[stream_id] = st.get();
    s->streams.push_back(std::move(st));
    return GDBG_OK;
}

int gdbg_server_stream_bytes(gdbg_server* s, uint64_t stream_id, uint64_t* bytes) {
    if (!s || !bytes) return sfail(GDBG_ERR_INVALID_ARG, "NULL argument");
    auto it = s->by_id.find(stream_id);
    if (it == s->by_id.end()) return sfail(GDBG_ERR_INVALID_ARG, "unknown stream");
    *bytes = it->second->footprint;
    return GDBG_OK;
}

int gdbg_server_submit(gdbg_server* s, uint64_t stream_id, const uint32_t* packed, uint64_t n_words,
                       const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers, double release_s,
                       uint64_t* n_new, uint64_t tag) {
    if (!s) return sfail(GDBG_ERR_INVALID_ARG, "NULL server");
    auto it = s->by_id.find(stream_id);
    if (it == s->by_id.end()) return sfail(GDBG_ERR_INVALID_ARG, "unknown stream");
    SStream* st = it->second;
    if (!offsets || (n_words && !packed)) return sfail(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (n_reads > st->max_reads || n_words > st->max_words)
        return sfail(GDBG_ERR_INVALID_ARG, "chunk larger than the stream's declared maximum");
    if (offsets[n_reads] > n_words * 16)
        return sfail(GDBG_ERR_INVALID_ARG, "offsets run past the packed words");
    if (n_kmers == UINT64_MAX) {
        n_kmers = 0;
        for (uint64_t r = 0; r < n_reads; ++r) {
            const uint64_t a = offsets[r], e = offsets[r + 1];
            if (e > a && e - a >= s->K) n_kmers += e - a - s->K + 1;
        }
    }
    std::lock_guard<std::mutex> lk(st->mu);
    if (st->finished) return sfail(GDBG_ERR_INVALID_ARG, "stream already finished");
    if (!st->queue.empty() && release_s < st->queue.back().release)
        return sfail(GDBG_ERR_INVALID_ARG, "release times of a stream must not decrease");
    st->queue.push_back({packed, n_words, offsets, n_reads, n_kmers, release_s, n_new, tag});
    ++st->submitted;
    s->submitted.fetch_add(1);
    return GDBG_OK;
}

int gdbg_server_finish(gdbg_server* s, uint64_t stream_id) {
    if (!s) return sfail(GDBG_ERR_INVALID_ARG, "NULL server");
    auto it = s->by_id.find(stream_id);
    if (it == s->by_id.end()) return sfail(GDBG_ERR_INVALID_ARG, "unknown stream");
    std::lock_guard<std::mutex> lk(it->second->mu);
    it->second->finished = true;
    return GDBG_OK;
}

int gdbg_server_start(gdbg_server* s) {
    if (!s) return sfail(GDBG_ERR_INVALID_ARG, "NULL server");
    if (s->started.exchange(true)) return sfail(GDBG_ERR_INVALID_ARG, "server already started");
    s->t0 = Clock::now();
    s->admitter = std::thread(admission_loop, s);
    for (uint32_t i = 0; i < s->n_dispatch; ++i) s->dispatchers.emplace_back(dispatch_loop, s, i);
    return GDBG_OK;
}

int gdbg_server_wait(gdbg_server* s, double timeout_s) {
    if (!s) return sfail(GDBG_ERR_INVALID_ARG, "NULL server");
    if (!s->started.load()) return sfail(GDBG_ERR_INVALID_ARG, "server not started");
    const double t_end = s->now() + timeout_s;
    for (;;) {
        bool all = true;
        for (auto& st : s->streams) {
            const int state = st->state.load();
            if (state == S_WAITING || state == S_ACTIVE) {
                all = false;
                break;
            }
        }
        if (all) return GDBG_OK;
        if (s->now() > t_end) return sfail(GDBG_ERR_DEVICE, "serving: wait timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

int gdbg_server_poll(gdbg_server* s, uint64_t* tags, double* latency_s, double* done_s, int32_t* ok,
                     uint64_t max, uint64_t* n_out) {
    if (!s || !n_out) return sfail(GDBG_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->done_mu);
    uint64_t n = 0;
    while (n < max && s->polled < s->completions.size()) {
        const Completion& c = s->completions[s->polled++];
        if (tags) tags[n] = c.tag;
        if (latency_s) latency_s[n] = c.latency;
        if (done_s) done_s[n] = c.done;
        if (ok) ok[n] = c.ok;
        ++n;
    }
    *n_out = n;
    return GDBG_OK;
}

int gdbg_server_stats(gdbg_server* s, gdbg_server_report* out) {
    if (!s || !out) return sfail(GDBG_ERR_INVALID_ARG, "NULL argument");
    std::memset(out, 0, sizeof *out);
    out->chunks_submitted = s->submitted.load();
    out->chunks_done = s->finished_chunks.load();
    out->chunks_failed = s->failed.load();
    out->kmers_done = s->kmers.load();
    out->streams = s->streams.size();
    out->streams_admitted = s->admitted.load();
    out->admission_waits = s->admission_waits.load();
    out->lazy_frees = s->lazy_frees.load();
    out->device_status = s->device_status.load();
    {
        std::lock_guard<std::mutex> lk(s->budget_mu);
        out->peak_hbm_bytes = s->peak;
    }
    std::lock_guard<std::mutex> lk(s->stat_mu);
    out->first_dispatch_s = s->first_dispatch;
    out->last_done_s = s->last_done;
    out->admit_s_max = s->admit_max;
    out->admit_s_total = s->admit_total;
    out->dispatch_s_max = s->dispatch_max;
    out->dispatch_s_total = s->dispatch_total;
    return GDBG_OK;
}

const char* gdbg_server_last_error(gdbg_server* s) {
    if (!s) return "";
    std::lock_guard<std::mutex> lk(s->stat_mu);
    return s->last_error.c_str();
}

int gdbg_server_destroy(gdbg_server* s) {
    if (!s) return GDBG_OK;
    s->stop.store(true);
    if (s->admitter.joinable()) s->admitter.join();
    // no stream may stay active without a dispatcher: drop what is queued
    for (auto& st : s->streams) {
        std::lock_guard<std::mutex> lk(st->mu);
        st->queue.clear();
        st->finished = true;
    }
    for (auto& t : s->dispatchers)
        if (t.joinable()) t.join();
    cudaSetDevice(s->device);
    for (auto& st : s->streams)
        if (st->state.load() != S_FREED && (st->g || !st->slots.empty())) free_stream_memory(st.get());
    delete s;
    return GDBG_OK;
}

}  // extern "C"
