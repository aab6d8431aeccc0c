/*
 * goetia_gb300 -- C ABI of the GB300 (sm_103a) dBG hot path.
 *
 * A drop-in for goetia's dBG<Storage, Shifter> hashing / insert / query /
 * neighbour-mask path (include/goetia/dbg.hh:39-438 and the layers under
 * it).  One opaque graph handle owns its device tables, its CUDA stream and
 * its scratch.  Every entry point returns GDBG_OK (0) or an error code; the
 * message of the last error on the calling thread is gdbg_last_error().
 * The reference throws C++ exceptions in the same places (see each entry).
 *
 * Reads enter in one of two forms:
 *   - strings (char*, len), the reference's own argument type, validated
 *     against DNA_SIMPLE ("ACGT");
 *   - packed batches: a 2-bit base stream (A=0 C=1 G=2 T=3, 16 bases per
 *     uint32_t, base j in bits 2*(j%16) of word j/16) plus n_reads+1 base
 *     offsets.  gdbg_pack_reads builds one from text reads.
 * k-mer outputs of a batch are flattened in read order; a read of length L
 * has L-K+1 k-mers, reads shorter than K have none.
 *
 * Calls on one handle must be serialised by the caller; different handles
 * may be used from different threads.  Functions named *_device take device
 * pointers and are asynchronous on `stream` (NULL = the handle's stream;
 * pass cudaStreamLegacy for the legacy default stream); all others take
 * host pointers and return when results are on the host.
 *
 * File:line citations are relative to the goetia source tree.
 */
#ifndef GOETIA_GB300_H
#define GOETIA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GDBG_OK 0
#define GDBG_ERR_INVALID_ARG 1
#define GDBG_ERR_SEQUENCE_LENGTH 2   /* SequenceLengthException, kmeriterator.hh:57-59,72-74 */
#define GDBG_ERR_INVALID_SEQUENCE 3  /* InvalidCharacterException, alphabets.hh:41-56 */
#define GDBG_ERR_CUDA 4
#define GDBG_ERR_OOM 5
#define GDBG_ERR_DEVICE 6            /* a device-side check failed (status word) */
#define GDBG_ERR_IO 7                /* GoetiaFileException, bitstorage.cc:151-307 */
#define GDBG_ERR_UNSUPPORTED 8

/* storage kinds: BitStorage (bitstorage.hh:93), ByteStorage
 * (bytestorage.hh:97), NibbleStorage (nibblestorage.hh:89) */
#define GDBG_BIT 0
#define GDBG_BYTE 1
#define GDBG_NIBBLE 2
/* shifter kinds: FwdLemireShifter / CanLemireShifter (hashshifter.hh:204-205) */
#define GDBG_FWD_LEMIRE 0
#define GDBG_CAN_LEMIRE 1

typedef struct gdbg_graph gdbg_graph;

const char* gdbg_last_error(void);
const char* gdbg_version(void);

/* ---- sizing and lifetime ---------------------------------------------- */

/* get_n_primes_near_x(n, x): the n largest odd primes below x, descending
 * (storage.hh:166-190).  *n_out may be < n when x is small. */
int gdbg_primes_near(uint32_t n, uint64_t x, uint64_t* out, uint32_t* n_out);

/* Storage::build(max_table, N) then dBG::build(storage, K)
 * (bitstorage.hh:69-71, dbg.hh:108-121).  Table sizes come from
 * gdbg_primes_near(n_tables, max_table). */
int gdbg_create(int storage, int shifter, uint16_t K, uint64_t max_table,
                uint16_t n_tables, gdbg_graph** out);
/* Storage(const std::vector<uint64_t>& tablesizes) (bitstorage.hh:73-81). */
int gdbg_create_sized(int storage, int shifter, uint16_t K, const uint64_t* sizes,
                      uint16_t n_tables, gdbg_graph** out);
int gdbg_destroy(gdbg_graph* g);
/* dBG::clone: a new graph with empty storage of the same shape (dbg.hh:128-131). */
int gdbg_clone(const gdbg_graph* g, gdbg_graph** out);
/* dBG::build(storage, K) on a storage that a graph already uses: the
 * reference's dBGs hold a shared_ptr<Storage> (dbg.hh:73, 97-101), so every
 * graph built on one storage inserts into and queries the same tables.  The
 * new handle shares g's device tables, table sizes and n_unique/n_occupied
 * counters (reference-counted: the tables are freed with the last handle);
 * its shifter, K, stream and scratch are its own.  Calls on handles that
 * share a storage must be ordered by the caller, like calls on one handle. */
int gdbg_share_storage(const gdbg_graph* g, int shifter, uint16_t K, gdbg_graph** out);
/* dBG::reset / Storage::reset: zero every table (bitstorage.cc:140-148).
 * Like the reference, the n_unique / n_occupied counters are kept. */
int gdbg_reset(gdbg_graph* g);
int gdbg_info(const gdbg_graph* g, int* storage, int* shifter, uint16_t* K, uint16_t* n_tables);
/* Storage::get_tablesizes (bitstorage.hh:160-163). */
int gdbg_get_tablesizes(const gdbg_graph* g, uint64_t* out);
/* Byte length of each table in the reference layout (size/8+1, size, size/2+1). */
int gdbg_table_bytes(const gdbg_graph* g, uint64_t* out);
/* dBG::get_raw (dbg.hh:224-226): all tables, concatenated, reference byte layout. */
int gdbg_get_tables(gdbg_graph* g, uint8_t* out, uint64_t out_len);
int gdbg_set_tables(gdbg_graph* g, const uint8_t* in, uint64_t in_len);
/* dBG::n_unique / n_occupied (dbg.hh:184-196). */
int gdbg_stats(gdbg_graph* g, uint64_t* n_unique, uint64_t* n_occupied);
/* dBG::save (dbg.hh:396-398) -> Storage::save: the OXLI v4 file of the
 * tables (bitstorage.cc:151-186, bytestorage.cc:480-521 with no bigcount
 * entries, nibblestorage.cc:132-166), byte-identical to the reference's for
 * the same tables.  Always a plain file: a ".gz" name is not compressed here
 * (the Python mirror compresses ByteStorage ".gz" files itself). */
int gdbg_save(gdbg_graph* g, const char* path);
/* dBG::load (dbg.hh:400-403) -> Storage::load (bitstorage.cc:188-307,
 * bytestorage.cc:172-290, nibblestorage.cc:168-250): checks signature,
 * version and file type (GDBG_ERR_IO with the reference's messages), takes
 * the file's table sizes (reallocating the tables when they differ) and
 * occupied-bin count; n_unique and K are kept, the file's ksize is returned
 * in *ksize (may be NULL).  The file is checked to be complete before any
 * state changes.  Byte files with use_bigcount set or bigcount entries are
 * GDBG_ERR_UNSUPPORTED (counts saturate at 255 here). */
int gdbg_load(gdbg_graph* g, const char* path, uint16_t* ksize);
/* BitStorage::update_from (bitstorage.cc:103-137): OR other's tables into
 * g's; n_occupied grows by the table-0 cells newly set, n_unique is kept.
 * Bit graphs only (GDBG_ERR_UNSUPPORTED otherwise, as the reference has no
 * Byte/Nibble update_from); different table sizes are GDBG_ERR_INVALID_ARG
 * ("both nodegraphs must have same table sizes").  Ordered after the work
 * queued on both handles' streams; returns when the merge is done. */
int gdbg_update_from(gdbg_graph* g, const gdbg_graph* other);
/* Use the caller's CUDA stream (cudaStream_t) for this handle; NULL restores
 * the handle's own stream. */
int gdbg_set_stream(gdbg_graph* g, void* stream);
int gdbg_synchronize(gdbg_graph* g);

/* ---- single sequences (the reference's per-read API) ------------------- */

/* HashShifter::hash(seq, K) on the first K symbols (hashshifter.hh:177-194);
 * fw/rc may be NULL (rc is 0 for the forward shifter). */
int gdbg_hash(gdbg_graph* g, const char* kmer, uint64_t len, uint64_t* value,
              uint64_t* fw, uint64_t* rc);
/* dBG::insert_sequence(seq, n_new) (dbg.hh:296-305): returns the k-mer count
 * in *n_kmers and the number of new k-mers in *n_new (either may be NULL). */
int gdbg_insert_sequence(gdbg_graph* g, const char* seq, uint64_t len,
                         uint64_t* n_kmers, uint64_t* n_new);
/* dBG::insert_and_query_sequence (dbg.hh:327-340): counts (len-K+1 entries)
 * get each k-mer's insert_and_query result in order; n_new (may be NULL) the
 * number of new k-mers.  Same limits as gdbg_insert_and_query_batch. */
int gdbg_insert_and_query_sequence(gdbg_graph* g, const char* seq, uint64_t len,
                                   int16_t* counts, uint64_t* n_new);
/* dBG::query_sequence(seq, counts, hashes) (dbg.hh:364-376); counts holds
 * len-K+1 entries, hashes may be NULL. */
int gdbg_query_sequence(gdbg_graph* g, const char* seq, uint64_t len, int16_t* counts,
                        uint64_t* hashes);
/* get_hash_iter over a sequence (dbg.hh:421-425): len-K+1 values; fw/rc may be NULL. */
int gdbg_hashes(gdbg_graph* g, const char* seq, uint64_t len, uint64_t* values,
                uint64_t* fw, uint64_t* rc);
/* Storage insert / query / insert_and_query of hash values, in order
 * (dbg.hh:144-177): n hashes; is_new / counts may be NULL. */
int gdbg_insert_hashes(gdbg_graph* g, const uint64_t* hashes, uint64_t n, uint8_t* is_new);
int gdbg_query_hashes(gdbg_graph* g, const uint64_t* hashes, uint64_t n, int16_t* counts);
/* Neighbour masks of every k-mer of seq: bit i = left extension "ACGT"[i]
 * present, bit 4+i = right extension present (set_cursor + in_degree /
 * out_degree, unitig_walker.hh:322-330, hashextender.hh:352-396).  A k-mer
 * is a decision k-mer iff popcount(mask & 15) > 1 or popcount(mask >> 4) > 1
 * (is_decision_kmer, unitig_walker.hh:1003-1023). */
int gdbg_neighbor_masks(gdbg_graph* g, const char* seq, uint64_t len, uint8_t* masks);

/* ---- packed batches, host buffers -------------------------------------- */

/* FastxParser<DNA_SIMPLE>::next policy (readers.hh:150-219): uppercase
 * acgt, drop (and count) reads holding any other symbol or shorter than
 * min_length.  packed needs total_len/16+1 words, offsets n_seqs+1. */
int gdbg_pack_reads(const char* seqs, const uint64_t* seq_offsets, uint64_t n_seqs,
                    uint32_t min_length, uint32_t* packed, uint64_t packed_words,
                    uint64_t* offsets, uint64_t* n_kept, uint64_t* n_skipped);
/* gdbg_pack_reads on the GPU: text reads and their n_seqs+1 byte offsets in
 * device memory, packed / offsets outputs in device memory (packed_words
 * words, zeroed here).  Kept bases in one call must stay below 2^32; a read
 * must be shorter than 2^31 bases.  Runs on `stream` (NULL = legacy default)
 * and returns when done, with the kept / skipped counts on the host. */
int gdbg_pack_reads_device(const char* seqs, const uint64_t* seq_offsets, uint64_t n_seqs,
                           uint32_t min_length, uint32_t* packed, uint64_t packed_words,
                           uint64_t* offsets, uint64_t* n_kept, uint64_t* n_skipped,
                           void* stream);
/* FastxParser<DNA_SIMPLE>::next called until the end (readers.hh:150-219,
 * over kseq, kseq.h:88-220) on FASTA / FASTQ text in device memory
 * (uncompressed, below 2^32 - 1 bytes), then gdbg_pack_reads_device's
 * policy and packing of the sequences.  Records are found in parallel for
 * the regular layouts -- four-line FASTQ records (one sequence line, one
 * quality line of its length); FASTA with sequences over any number of
 * lines and no line starting with '+' -- and the result is then what kseq
 * gives; other text (several quality lines, junk before the first header,
 * blank lines after a FASTQ record ...) is GDBG_ERR_UNSUPPORTED, naming the
 * first line that breaks the layout, for the caller to parse on the host.
 * stats: [0] reads kept, [1] reads dropped, [2] records parsed
 * (FastxParser::n_parsed), [3] FastxParser::n_skipped (a read both invalid
 * and shorter than min_length counts twice).  offsets needs stats[2] + 1
 * entries (GDBG_ERR_INVALID_ARG with stats[2] set otherwise), packed the
 * sequence bytes / 16 + 1 words (n_bytes / 16 + 1 always suffices).  Runs
 * on `stream` and returns when done.  Its scratch, and the device packer's,
 * comes from a memory pool of the library's own per device that keeps up
 * to 2 GiB reserved between calls (for the process's lifetime). */
int gdbg_parse_fastx_device(const char* text, uint64_t n_bytes, uint32_t min_length,
                            uint32_t* packed, uint64_t packed_words, uint64_t* offsets,
                            uint64_t offsets_cap, uint64_t* stats, void* stream);
/* 2-bit codes (one byte each, values 0..3) to the packed stream. */
int gdbg_pack_codes(const uint8_t* codes, uint64_t n, uint32_t* packed);

/* insert_sequence(seq, n_new) for every read in batch order (dbg.hh:296-305
 * called by InserterProcessor, processors.hh:304-331).  n_new (per read,
 * may be NULL) equals the reference's sequential result exactly. */
int gdbg_insert_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                      const uint64_t* offsets, uint64_t n_reads, uint64_t* n_new,
                      uint64_t* n_kmers);
/* query_sequence for every read (dbg.hh:349-362): flattened counts. */
int gdbg_query_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                     const uint64_t* offsets, uint64_t n_reads, int16_t* counts);
/* insert_and_query_sequence for every read, in batch order (dbg.hh:327-340;
 * also the counts of insert_sequence(seq, hashes, counts), dbg.hh:249-265):
 * per k-mer 1 if it was new, else the storage's count right after its own
 * insert (bytestorage.cc:142-150, nibblestorage.cc:103-109; always 1 for
 * BitStorage, bitstorage.cc:78-84), exactly as sequential calls would
 * return.  n_new (may be NULL) gets the per-read new counts.  Needs at most
 * 8 tables of at most 2^32 cells in total (GDBG_ERR_UNSUPPORTED otherwise). */
int gdbg_insert_and_query_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                                const uint64_t* offsets, uint64_t n_reads, int16_t* counts,
                                uint64_t* n_new);
/* get_hash_iter for every read: flattened values (and fw/rc, may be NULL). */
int gdbg_hashes_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                      const uint64_t* offsets, uint64_t n_reads, uint64_t* values,
                      uint64_t* fw, uint64_t* rc);
/* Neighbour masks for every k-mer of every read (find_decision_kmers,
 * unitig_walker.hh:1025-1045, with the per-k-mer mask kept). */
int gdbg_neighbor_masks_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                              const uint64_t* offsets, uint64_t n_reads, uint8_t* masks);

/* The compactor's per-k-mer query (StreamingCompactor::find_new_segments,
 * compactor.hh:346-466), every read against the storage as it is (the
 * compactor inserts a sequence's k-mers only after this query):
 *   flags bit 0: new   -- query() == 0 (compactor.hh:364)
 *   flags bit 1: seen  -- the hash is already in the read's new-k-mer set
 *                         at this position (compactor.hh:365)
 *   masks: the 8-bit neighbour mask (as gdbg_neighbor_masks) where a
 *          neighbour is present when query() != 0 or it is one of the
 *          read's new k-mers (filter_nodes with extras, unitig_walker.hh:
 *          457-469; get_decision_neighbors(..., union_nodes), :1054-1083).
 * Decision k-mers of the compactor's segments are those whose mask has more
 * than one left or more than one right neighbour. */
int gdbg_compactor_sequence(gdbg_graph* g, const char* seq, uint64_t len, uint8_t* flags,
                            uint8_t* masks);
int gdbg_compactor_batch(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                         const uint64_t* offsets, uint64_t n_reads, uint8_t* flags,
                         uint8_t* masks);

/* ---- packed batches, device buffers (asynchronous) --------------------- */

/* Same as gdbg_insert_batch with device pointers, asynchronous on `stream`.
 * packed_words bounds the packed stream: reads whose offsets decrease or run
 * past 16*packed_words are rejected on the device (GDBG_ERR_DEVICE at the next
 * synchronising call).  n_kmers_hint is the batch's k-mer count when the
 * caller knows it (saves one device-to-host read), else UINT64_MAX.  n_new
 * (device, one uint64 per read) may be NULL. */
int gdbg_insert_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                             const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                             uint64_t* n_new, void* stream);
/* gdbg_insert_batch_device fed from host buffers, asynchronously: the copy
 * of packed/offsets to the handle's staging buffers, the insert and the copy
 * of the per-read new counts back to n_new (may be NULL) are all queued on
 * `stream`; the call returns at once.  The host buffers must stay untouched
 * until the stream has passed this call (record an event after it); with
 * pinned buffers the copies overlap other streams' work.  n_kmers is the
 * batch's k-mer count (or an upper bound), or UINT64_MAX to have the call
 * count it from the host offsets.  Calls on one handle reuse its staging
 * buffers in stream order; the copies of a batch of 2^20 packed words or
 * more go to one of two staging slots on the handle's copy stream, so they
 * overlap the kernels of the batch queued before it. */
int gdbg_insert_batch_async(gdbg_graph* g, const uint32_t* packed, uint64_t n_words,
                            const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers,
                            uint64_t* n_new, void* stream);
int gdbg_query_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                            const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                            int16_t* counts, void* stream);
int gdbg_insert_and_query_batch_device(gdbg_graph* g, const uint32_t* packed,
                                       uint64_t packed_words, const uint64_t* offsets,
                                       uint64_t n_reads, uint64_t n_kmers_hint, int16_t* counts,
                                       uint64_t* n_new, void* stream);
int gdbg_hashes_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                             const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                             uint64_t* values, uint64_t* fw, uint64_t* rc, void* stream);
int gdbg_compactor_batch_device(gdbg_graph* g, const uint32_t* packed, uint64_t packed_words,
                                const uint64_t* offsets, uint64_t n_reads, uint64_t n_kmers_hint,
                                uint8_t* flags, uint8_t* masks, void* stream);
int gdbg_neighbor_masks_batch_device(gdbg_graph* g, const uint32_t* packed,
                                     uint64_t packed_words, const uint64_t* offsets,
                                     uint64_t n_reads, uint64_t n_kmers_hint, uint8_t* masks,
                                     void* stream);

/* ---- tuning and diagnostics ------------------------------------------- */

/* Insert schedule: k-mers per window (<= 2^20; each window is a probe pass
 * then a commit pass) and k-mers per thread of the windowed path (4 or 8).
 * 0 keeps a value. */
int gdbg_set_insert_schedule(gdbg_graph* g, uint32_t window_kmers, uint32_t kmers_per_thread);
/* Read-batch insert implementation; all give identical results.
 *   PERSISTENT  one cooperative launch per batch, per-k-mer table access;
 *               its blocks wait on each other at grid barriers (bounded), so
 *               do not run two such inserts concurrently on different streams
 *   WINDOWED    one probe and one commit launch per window
 *   BUCKETED    records partitioned by table region with two unstable digit
 *               passes, each region applied in shared memory independently of
 *               record order (large batches on tables far beyond L2); falls
 *               back to BUCKETED_ORDERED outside its limits (more than
 *               2^17 buckets or regions above 64 KB)
 *   BUCKETED_ORDERED  the same with stable digit passes and regions applied
 *               in k-mer order (also the path of insert_and_query batches)
 *   AUTO        BUCKETED for batches of >= 4M k-mers on >= 256 MB of tables,
 *               else WINDOWED (default) */
#define GDBG_PATH_PERSISTENT 0
#define GDBG_PATH_WINDOWED 1
#define GDBG_PATH_BUCKETED 2
#define GDBG_PATH_AUTO 3
#define GDBG_PATH_BUCKETED_ORDERED 4
int gdbg_set_insert_path(gdbg_graph* g, int path);
/* Cells per bucket of the bucketed paths as log2 (0 = default: 32 KB of
 * table per bucket for BUCKETED, 64 KB for BUCKETED_ORDERED). */
int gdbg_set_bucket_bits(gdbg_graph* g, uint32_t log2_cells);
int gdbg_get_insert_schedule(const gdbg_graph* g, uint32_t* window_kmers,
                             uint32_t* kmers_per_thread);
/* Device status word (GDBG_ERR_* device bits); cleared by reading. */
int gdbg_device_status(gdbg_graph* g, uint32_t* status);
/* Poll limits of the bounded device waits on this handle: barrier_polls for
 * a grid-barrier wait of the PERSISTENT insert, copy_polls for the first wait
 * on each shared-memory bulk copy of the BUCKETED insert (0 = the default,
 * 2^24 polls, a second or two).  A wait that runs out sets a device status
 * bit (4 = barrier timeout, 16 = bulk-copy timeout), its kernel returns
 * without finishing the batch, and the next synchronising call reports
 * GDBG_ERR_DEVICE; the tables are then partly updated (gdbg_reset clears
 * them).  Before a block gives up it still waits, with the default limit,
 * for its own copies in flight.  A diagnostic with no counterpart in the
 * reference: it lets a test drive those error paths without a GPU fault. */
int gdbg_set_wait_limits(gdbg_graph* g, uint32_t barrier_polls, uint32_t copy_polls);
/* Grow the graph's batch and windowed-insert scratch for batches of up to
 * max_reads reads and max_kmers k-mers now, so later inserts within that
 * size allocate nothing. */
int gdbg_reserve(gdbg_graph* g, uint64_t max_reads, uint64_t max_kmers);
/* Grow the host-call staging buffers for batches of up to max_words packed
 * words and max_reads reads (gdbg_insert_batch_async and the host-buffer
 * batch calls then allocate nothing up to that size). */
int gdbg_reserve_staging(gdbg_graph* g, uint64_t max_words, uint64_t max_reads);
/* Per-stage timing: when on, every stage of a batch insert is bracketed by
 * CUDA events on its stream.  gdbg_stage_times synchronises, returns the
 * accumulated milliseconds and launch counts per stage (names comma-separated
 * in `names`) and resets the totals. */
int gdbg_set_profiling(gdbg_graph* g, int on);
int gdbg_stage_times(gdbg_graph* g, char* names, uint64_t names_len, double* total_ms,
                     uint64_t* launches, uint32_t max_stages, uint32_t* n_stages);
/* Kernel launches issued by this handle since creation. */
int gdbg_launch_count(const gdbg_graph* g, uint64_t* launches);

/* ---- serving: many streams, one graph each, continuous batching ------- */

/* The reference's streaming driver (goetia/processors.py:39-498,
 * AsyncSequenceProcessor; each chunk is InserterProcessor::process_sequence
 * per read, processors.hh:304-331) serves one sample at a time.  A server
 * serves many at once on the current device: each declared stream gets its
 * own graph (tables, windowed insert, own CUDA stream) when its first chunk
 * is due and its footprint fits hbm_budget (streams are admitted in the order
 * their next chunks are due; a drained stream returns its share at once and
 * its device memory is freed when an admission needs the room).  Native
 * dispatcher threads (dispatch_threads of them) copy each released chunk into
 * pinned staging and insert it asynchronously, up to `depth` chunks of a
 * stream in flight, so chunks of different streams overlap on the GPU while
 * each stream's chunks apply in order; per-chunk new counts equal inserting
 * the stream's reads one by one (dbg.hh:296-305).  Latency of a chunk =
 * completion time - release time.
 *
 * Use: create; declare every stream (gdbg_server_stream: table size and its
 * largest chunk); submit chunks (host buffers that stay valid until the chunk
 * completes; n_new = host output of n_reads counts, may be NULL; release_s =
 * seconds after gdbg_server_start, non-decreasing per stream; n_kmers =
 * UINT64_MAX to count them here) and mark each stream finished; start; wait;
 * poll the completions (tag, latency, completion time, ok); destroy.  Chunks
 * may also be submitted after start.  A stream whose footprint exceeds the
 * budget is rejected when declared (GDBG_ERR_OOM). */
typedef struct gdbg_server gdbg_server;
typedef struct {
    uint64_t chunks_submitted, chunks_done, chunks_failed, kmers_done;
    uint64_t streams, streams_admitted, admission_waits, lazy_frees, peak_hbm_bytes;
    double first_dispatch_s, last_done_s;   /* seconds after start */
    double admit_s_max, admit_s_total;      /* graph creation on admission */
    double dispatch_s_max, dispatch_s_total;/* host time per chunk dispatch */
    uint32_t device_status;                 /* OR of the streams' device status bits */
} gdbg_server_report;
int gdbg_server_create(int storage, int shifter, uint16_t K, uint16_t n_tables,
                       uint64_t hbm_budget, uint32_t depth, uint32_t dispatch_threads,
                       gdbg_server** out);
int gdbg_server_stream(gdbg_server* s, uint64_t stream_id, uint64_t max_table,
                       uint64_t max_chunk_reads, uint64_t max_chunk_words);
/* The HBM budget share of a declared stream (its admission footprint). */
int gdbg_server_stream_bytes(gdbg_server* s, uint64_t stream_id, uint64_t* bytes);
int gdbg_server_submit(gdbg_server* s, uint64_t stream_id, const uint32_t* packed,
                       uint64_t n_words, const uint64_t* offsets, uint64_t n_reads,
                       uint64_t n_kmers, double release_s, uint64_t* n_new, uint64_t tag);
int gdbg_server_finish(gdbg_server* s, uint64_t stream_id);
int gdbg_server_start(gdbg_server* s);
/* Until every declared stream has drained (GDBG_ERR_DEVICE after timeout_s). */
int gdbg_server_wait(gdbg_server* s, double timeout_s);
/* Completions not yet polled, in completion order (up to max). */
int gdbg_server_poll(gdbg_server* s, uint64_t* tags, double* latency_s, double* done_s,
                     int32_t* ok, uint64_t max, uint64_t* n_out);
int gdbg_server_stats(gdbg_server* s, gdbg_server_report* out);
/* Message of the server's last failure (admission or dispatch), or "". */
const char* gdbg_server_last_error(gdbg_server* s);
/* Stops the threads (queued chunks are dropped), frees every stream. */
int gdbg_server_destroy(gdbg_server* s);

/* ---- insert without device allocation -------------------------------- */

/* Limits of gdbg_insert_batch_noalloc (sizes of its static scratch). */
#define GDBG_NOALLOC_MAX_READS 131072u
#define GDBG_NOALLOC_MAX_TASKS 1048576u   /* packed_words/2 + n_reads must not exceed it */
#define GDBG_NOALLOC_MAX_TABLES 8u
#define GDBG_NOALLOC_SCRATCH_BYTES 17825792u

/* Word offset of each table (and the total, entry n_tables) in the table
 * buffer gdbg_insert_batch_noalloc works on: table i holds the reference's
 * bytes (size/8+1, size or size/2+1) padded to a multiple of 256 bytes. */
int gdbg_noalloc_table_layout(int storage, const uint64_t* sizes, uint16_t n_tables,
                              uint64_t* word_offsets);

/* No counterpart in the reference: it exists for callers that cannot
 * allocate device memory -- a framework that hands out all GPU memory from
 * its own fixed pool, or a latency-critical loop that must not pay the
 * device-wide synchronisation of cudaMalloc/cudaFree.  Inserts one packed
 * batch (device pointers, as gdbg_insert_batch_device) into caller-owned
 * tables (`tables`, device, laid out by gdbg_noalloc_table_layout, zeroed
 * by the caller before first use) with the same exact results, and calls no
 * cudaMalloc, cudaFree or allocating library routine.  Its scratch is a
 * static device array of GDBG_NOALLOC_SCRATCH_BYTES that every GPU loading
 * this library holds until exit; batches beyond GDBG_NOALLOC_MAX_READS reads
 * or GDBG_NOALLOC_MAX_TASKS warp tasks, or with more than
 * GDBG_NOALLOC_MAX_TABLES tables, are rejected with GDBG_ERR_INVALID_ARG.
 * The first call on a device looks the array up and clears it: make that
 * call before any stream capture.  Calls share the array; calls that overlap
 * on the GPU race and must be serialised by the caller.  n_new (device, one
 * uint64 per read) may be NULL.  stats (device, 3 x uint64) receives the
 * call's n_unique and n_occupied increments and the device status bits
 * (non-zero = a device-side check failed: 1 CAS cap, 2 claims map full,
 * 4 barrier timeout, 8 bad read offsets); the call then returns at once.
 * With stats NULL the call waits for the insert on `stream` and returns
 * GDBG_ERR_DEVICE when a device-side check failed, so no failure goes
 * unreported.  Offsets are checked on the device, as by
 * gdbg_insert_batch_device: a read whose offsets decrease or run past
 * 16*packed_words counts as zero k-mers, the batch's other reads are still
 * inserted, and status bit 8 reports it (gdbg_insert_batch, with host
 * buffers, rejects such a batch before touching any table). */
int gdbg_insert_batch_noalloc(int storage, int shifter, uint16_t K, const uint64_t* sizes,
                              uint16_t n_tables, uint32_t* tables, const uint32_t* packed,
                              uint64_t packed_words, const uint64_t* offsets, uint64_t n_reads,
                              uint64_t* n_new, uint64_t* stats, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GOETIA_GB300_H */
