// Host-side launchers.  Each storage translation unit defines the
// launch_*<STORAGE> specialisations; the API code dispatches on the
// handle's storage kind.
#pragma once
#include <cuda_runtime.h>

#include "gdbg_types.h"

#include <string>

namespace gdbg {

// Record the message behind a failing status for gdbg_last_error(); returns code.
int report_error(int code, const std::string& msg);

struct LaunchShape {
    bool canonical;
    int kmers_per_thread;   // 4 or 8
    int n_tables;           // 4 uses the unrolled kernels, others the generic ones
};

// pass 0 = probe, 1 = commit, 2 = both in one block (n_threads <= SMALL_BLOCK),
// 3 = both in one block with one k-mer per thread (n_threads = the window's
// k-mers <= SMALL_BLOCK); hashes != nullptr selects the hash-array source
template <int STORAGE>
cudaError_t launch_insert_pass(int pass, const LaunchShape& s, uint64_t n_threads,
                               cudaStream_t st, const BatchView& b, const uint64_t* hashes,
                               const HashParams& hp, const TableParams& tp,
                               const WindowParams& w);

// One read's insert in one CTA (k_insert_read, at most 8 tables): n_new[0]
// gets the read's new k-mers added; counters[0] / [1] n_unique / n_occupied;
// done (may be null) gets (seq << 32) | the device status word as the insert's
// last write.  set_attr: the kernel's shared-memory opt-in (once per device).
template <int STORAGE>
cudaError_t launch_insert_read(bool canonical, bool set_attr, cudaStream_t st, const BatchView& b,
                               const HashParams& hp, const TableParams& tp, uint64_t* n_new,
                               unsigned long long* counters, uint32_t* err, uint64_t* done,
                               uint32_t seq);
constexpr int READ_INSERT_MAXNT = 8;

struct PersistParams;

// Persistent cooperative insert of a whole read batch (gdbg_persist.cuh).
// max_tasks bounds the batch's warp tasks; *grid_used gets the block count.
template <int STORAGE>
cudaError_t launch_insert_persistent(const LaunchShape& s, uint64_t max_tasks, cudaStream_t st,
                                     const BatchView& b, const HashParams& hp,
                                     const TableParams& tp, const PersistParams& pp,
                                     int* grid_used);

template <int STORAGE>
cudaError_t launch_query(const LaunchShape& s, uint64_t n_total, cudaStream_t st,
                         const BatchView& b, const uint64_t* hashes, const HashParams& hp,
                         const TableParams& tp, int16_t* counts, uint64_t* values);

template <int STORAGE>
cudaError_t launch_masks(const LaunchShape& s, cudaStream_t st, const BatchView& b,
                         const HashParams& hp, const TableParams& tp, uint8_t* masks);

cudaError_t launch_hashes(bool canonical, cudaStream_t st, const BatchView& b,
                          const HashParams& hp, uint64_t* values, uint64_t* fw, uint64_t* rc);

// Bucketed insert (gdbg_bucket.cu / gdbg_bucket.cuh).
struct BucketParams;
cudaError_t launch_bucket_emit(bool canonical, cudaStream_t st, const BatchView& b,
                               const HashParams& hp, const TableParams& tp, const BucketParams& bp);
cudaError_t launch_bucket_hist(uint32_t n_tiles, cudaStream_t st, const BucketParams& bp);
cudaError_t launch_bucket_scatter(bool last, uint32_t n_tiles, cudaStream_t st,
                                  const BucketParams& bp, uint32_t* start);
cudaError_t launch_bucket_starts_fix(cudaStream_t st, const BucketParams& bp, uint32_t* start);
uint64_t bucket_tile_records();
// vals != nullptr (Byte/Nibble): also store each record's post-insert value
// for insert_and_query (vals[table * kmer_cap + k-mer]).
cudaError_t launch_bucket_apply(int storage, const TableParams& tp, const BucketParams& bp,
                                const uint64_t* recs, const uint32_t* start, uint32_t* new_bits,
                                unsigned long long* counters, uint8_t* vals, cudaStream_t st);
// Per-k-mer insert_and_query counts from vals and the new-k-mer bitmask.
cudaError_t launch_iq_counts(const uint8_t* vals, uint64_t cap, uint32_t n_tables,
                             const uint32_t* new_bits, const uint64_t* total, int16_t* counts,
                             bool presence, cudaStream_t st);
cudaError_t launch_bucket_read_new(const uint64_t* kofs, uint64_t n_reads, const uint32_t* new_bits,
                                   uint64_t* n_new, unsigned long long* counters, cudaStream_t st);
uint64_t scan32_partials_needed(uint64_t n);
// Exclusive scan of n uint32.  With a gate, the kernels return at once
// unless *gate is non-zero when they run.
cudaError_t launch_scan32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* partials,
                          cudaStream_t st, const uint32_t* gate = nullptr);

// Batch preparation (gdbg_batch.cu): per-read k-mer prefix and tile map.
// Validates offsets (non-decreasing, within max_bases) on the device; a bad
// read counts as zero k-mers and sets GDBG_ERR_BAD_OFFSETS in *err.
cudaError_t launch_kmer_prefix(const uint64_t* offsets, uint64_t n_reads, uint32_t K,
                               uint64_t max_bases, uint64_t* partials, uint64_t* kofs,
                               uint64_t* tofs, uint32_t* err, cudaStream_t st, int* launches);
// task_read[t] for every warp task t < cap (tasks: 32 k-mers of one read).
cudaError_t launch_task_map(const uint64_t* tofs, uint64_t n_reads, uint64_t cap,
                            uint32_t* task_read, cudaStream_t st);
cudaError_t launch_tile_map(const uint64_t* kofs, uint64_t n_reads, uint64_t n_tiles,
                            uint32_t* tile_read, cudaStream_t st);

// Segmented bucketed insert (gdbg_sort.cu / gdbg_sort.cuh).
// segments [seg0, seg0 + n_seg) of the batch (clipped to sp.nseg1)
cudaError_t launch_sp_emit(bool canonical, cudaStream_t st, const BatchView& b, const HashParams& hp,
                           const TableParams& tp, const SortParams& sp, uint64_t* rout,
                           uint32_t seg0, uint32_t n_seg);
// The emit and pass 1 fused (four tables), into the reserved pass-1 layout
// that k_sp_groups sizes; segments [seg0, seg0 + n_seg) of the batch.
cudaError_t launch_sp_groups(cudaStream_t st, const SortParams& sp);
cudaError_t launch_sp_emit_part(bool canonical, cudaStream_t st, const BatchView& b, const HashParams& hp,
                                const TableParams& tp, const SortParams& sp, uint64_t* rout,
                                uint32_t seg0, uint32_t n_seg);
// Partition passes: pass 1, pass 2 into the reserved layout, pass 2 into the
// counted layout (a no-op when the reserved one was made and held).
enum { SP_PASS1 = 0, SP_PASS2_RESERVED = 1, SP_PASS2_COUNTED = 2 };
cudaError_t launch_sp_part(int pass, cudaStream_t st, const SortParams& sp, const uint64_t* rin,
                           uint64_t* rout);
cudaError_t launch_sp_plan(cudaStream_t st, const SortParams& sp);
cudaError_t launch_sp_hist2(cudaStream_t st, const SortParams& sp, const uint64_t* rin);
// Record range [start[b], end[b]) of every bucket.
cudaError_t launch_sp_starts(cudaStream_t st, const SortParams& sp, uint32_t* start, uint32_t* end);
cudaError_t launch_sp_apply(int storage, const TableParams& tp, const SortParams& sp,
                            const uint64_t* recs, const uint32_t* start, const uint32_t* end,
                            uint32_t* new_bits, unsigned long long* counters, cudaStream_t st);
size_t sp_apply_smem_bytes(int storage, uint32_t fs);

// Stream-ordered scratch (free with cudaFreeAsync) from the library's own
// pool of the current device, which keeps up to 2 GiB between calls
// (gdbg_pack_device.cu).
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t st);

// Device packing of text reads (gdbg_pack_device.cu): read r =
// seqs[starts[r], ends[r]); out[0] kept, [1] dropped, [2] dropped reads
// both invalid and shorter than min_length.  Synchronous.
int pack_device_run(const char* seqs, const uint64_t* starts, const uint64_t* ends, uint64_t n_seqs,
                    uint32_t min_length, uint32_t* packed, uint64_t packed_words,
                    uint64_t* offsets, uint64_t out[3], cudaStream_t st);

// Compactor query (gdbg_compactor.cu): per k-mer new / seen flags and the
// neighbour masks over the storage plus each read's new k-mers.  keys /
// minpos hold compactor_slots() entries set to all ones, allones n_reads.
cudaError_t launch_compactor(int storage, const LaunchShape& s, cudaStream_t st, const BatchView& b,
                             const HashParams& hp, const TableParams& tp, uint64_t* keys,
                             uint32_t* minpos, uint32_t* allones, uint8_t* flags, uint8_t* masks,
                             uint32_t* err);
uint64_t compactor_slots(uint64_t n_kmers, uint64_t n_reads);

// OR-merge of two identically laid out table allocations (n_words, a
// multiple of 4); cells newly set in the first count_words words are added
// to *occupied.
cudaError_t launch_or_merge(uint32_t* dst, const uint32_t* src, uint64_t n_words,
                            uint64_t count_words, unsigned long long* occupied, cudaStream_t st);

}  // namespace gdbg
