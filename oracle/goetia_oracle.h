/*
 * CPU oracle for the goetia dBG hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (sequential rolling
 * cyclic hash, Bit/Byte/Nibble storages, dBG insert/query, neighbour masks,
 * and the FASTA/FASTQ reader in front of them: kseq and FastxParser).
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark use
 * it, as the checker; the product path never links or calls it.
 *
 * Parity is pinned two ways: the K=27 known-answer hash from the reference's
 * tests (tests/test_hashing.py:15-19), and golden fixtures generated by the
 * reference's own C++ objects (oracle/Makefile + oracle/ref_driver.cc, and
 * oracle/ref_fastx.cc for the reader).
 *
 * Read encoding (shared with the GPU library): bases are 2-bit codes
 * A=0 C=1 G=2 T=3, packed 16 per uint32_t little-endian (base j is bits
 * 2*(j%16)..2*(j%16)+1 of word j/16).  A batch of reads is a packed base
 * stream plus n_reads+1 base offsets.
 */
#ifndef GOETIA_ORACLE_H
#define GOETIA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BIT = 0, ORC_BYTE = 1, ORC_NIBBLE = 2 };

typedef struct orc_storage orc_storage;

/* Hashing */
void     orc_symbol_table(uint64_t out[4]);
void     orc_hash_codes(const uint8_t* codes, uint64_t len, uint16_t K,
                        uint64_t* fw, uint64_t* rc);
uint32_t orc_primes(uint32_t n, uint64_t x, uint64_t* out);

/* Storage */
orc_storage* orc_storage_new(int kind, const uint64_t* sizes, int n_tables);
void         orc_storage_free(orc_storage* s);
int          orc_n_tables(const orc_storage* s);
uint64_t     orc_table_bytes(const orc_storage* s, int i);
const uint8_t* orc_table(const orc_storage* s, int i);
void         orc_stats(const orc_storage* s, uint64_t* n_unique, uint64_t* n_occupied);
int          orc_insert(orc_storage* s, uint64_t h);
int16_t      orc_query(const orc_storage* s, uint64_t h);
int16_t      orc_insert_and_query(orc_storage* s, uint64_t h);
void         orc_reset(orc_storage* s);

/* Read batches (packed 2-bit stream + base offsets). k-mer outputs are
 * flattened in read order; reads shorter than K contribute none. */
uint64_t orc_count_kmers(uint16_t K, const uint64_t* offsets, uint64_t n_reads);
void     orc_hash_reads(int canonical, uint16_t K, const uint32_t* packed,
                        const uint64_t* offsets, uint64_t n_reads,
                        uint64_t* val, uint64_t* fw, uint64_t* rc);
uint64_t orc_insert_reads(orc_storage* s, int canonical, uint16_t K,
                          const uint32_t* packed, const uint64_t* offsets,
                          uint64_t n_reads, uint64_t* n_new);
void     orc_insert_and_query_reads(orc_storage* s, int canonical, uint16_t K,
                                    const uint32_t* packed, const uint64_t* offsets,
                                    uint64_t n_reads, int16_t* counts);
void     orc_query_reads(const orc_storage* s, int canonical, uint16_t K,
                         const uint32_t* packed, const uint64_t* offsets,
                         uint64_t n_reads, int16_t* counts);
/* compactor.hh:346-466: per k-mer new / seen flags and neighbour masks over
 * the storage plus the read's new k-mers. */
void     orc_compactor_reads(const orc_storage* s, int canonical, uint16_t K,
                             const uint32_t* packed, const uint64_t* off, uint64_t n,
                             uint8_t* flags, uint8_t* masks);
void     orc_decision_masks(const orc_storage* s, int canonical, uint16_t K,
                            const uint32_t* packed, const uint64_t* offsets,
                            uint64_t n_reads, uint8_t* masks);
/* Throughput-only multi-threaded insert (reads round-robin over threads into
 * one shared storage with atomic cell updates).  Final table bytes equal the
 * sequential result; new-k-mer counts are order dependent and not reported. */
uint64_t orc_insert_reads_mt(orc_storage* s, int canonical, uint16_t K,
                             const uint32_t* packed, const uint64_t* offsets,
                             uint64_t n_reads, int n_threads);

/* min(255, number of inserts hitting each cell [lo[j], lo[j] + width) of
 * table tables[j]) over every k-mer of the batch, ADDED to out (n_sel x
 * width bytes, saturating at 255), so calls over consecutive batches
 * accumulate.  Order independent: the final value of a saturating cell. */
int      orc_count_cells(int canonical, uint16_t K, const uint32_t* packed,
                         const uint64_t* offsets, uint64_t n_reads, const uint64_t* sizes,
                         const int* tables, int n_sel, const uint64_t* lo, uint64_t width,
                         uint8_t* out, int n_threads);

/* FASTX parser policy for DNA_SIMPLE: uppercase acgt, drop any read holding
 * another symbol, drop reads shorter than min_length. */
int64_t  orc_pack_ascii(const char* seqs, const uint64_t* seq_offsets, uint64_t n_seqs,
                        uint32_t min_length, uint32_t* packed, uint64_t* offsets,
                        uint64_t* n_skipped);

/* FastxParser<DNA_SIMPLE>::next over FASTA/FASTQ text held in memory (kseq
 * grammar, kseq.h:88-220; parser policy, readers.hh:150-219), called until
 * the stream ends.  The kept reads' sequences (upper-cased) go to seq_out
 * (seq_cap bytes) with their seq_off[0..kept] offsets (rec_cap + 1 entries).
 * stats: [0] n_parsed, [1] n_skipped (FastxParser's counters: a read that is
 * both invalid and shorter than min_length counts twice), [2] reads
 * dropped, [3] the record at which kseq reported differing sequence and
 * quality lengths.  Returns the kept count, -2 at that InvalidRead (reads
 * before it are kept), -5 when seq_cap or rec_cap is too small. */
int64_t  orc_parse_fastx(const char* text, uint64_t n, uint32_t min_length, char* seq_out,
                         uint64_t seq_cap, uint64_t* seq_off, uint64_t rec_cap,
                         uint64_t stats[4]);

#ifdef __cplusplus
}
#endif
#endif
