/*
 * CPU oracle for the goetia dBG hot path -- TEST INFRASTRUCTURE ONLY.
 * See goetia_oracle.h for scope and encoding.  Every function restates the
 * reference's sequential algorithm; file:line citations are relative to the
 * goetia source tree.
 */
#define _GNU_SOURCE
#include "goetia_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* CharacterHash::hashvalues entries for 'A', 'C', 'G', 'T'
 * (include/goetia/hashing/rollinghash/characterhash.h:49-56; Lemire's
 * rollinghashcpp, Apache-2.0), indexed by 2-bit code. */
static const uint64_t SYM[4] = {
    16664410744025174816ull, /* 'A' = 65 */
    15956807086001210932ull, /* 'C' = 67 */
    9404339731978646439ull,  /* 'G' = 71 */
    836480985777824379ull,   /* 'T' = 84 */
};

void orc_symbol_table(uint64_t out[4]) { memcpy(out, SYM, sizeof(SYM)); }

/* ---- CyclicHash<uint64_t> (rollinghash/cyclichash.h:24-138) ------------ */

static inline uint64_t rotl64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x << r) | (x >> (64u - r)) : x;
}

typedef struct { uint64_t h; unsigned myr; } cyclic;

static inline void cyc_reset(cyclic* c, uint16_t K) { c->h = 0; c->myr = K % 64u; }
/* eat: fastleftshift1 then xor (cyclichash.h:105-108) */
static inline void cyc_eat(cyclic* c, int sym) { c->h = rotl64(c->h, 1) ^ SYM[sym]; }
/* update(out, in): rotl1(h) ^ rotl_{n mod 64}(T[out]) ^ T[in] (cyclichash.h:85-92) */
static inline void cyc_update(cyclic* c, int out, int in) {
    c->h = rotl64(c->h, 1) ^ rotl64(SYM[out], c->myr) ^ SYM[in];
}
/* reverse_update(out, in): h ^= rotl_n(T[out]) ^ T[in]; h = rotr1(h) (cyclichash.h:96-101) */
static inline void cyc_reverse_update(cyclic* c, int out, int in) {
    uint64_t x = c->h ^ rotl64(SYM[out], c->myr) ^ SYM[in];
    c->h = (x >> 1) | (x << 63);
}

/* DNA_SIMPLE::complement on codes (alphabets.hh:132-144) */
static inline int comp(int c) { return 3 - c; }

/* ---- LemireShifterPolicy fw / canonical (rollinghashshifter.hh) -------- */

typedef struct { cyclic fw, rc; int canonical; uint16_t K; } shifter;

static void sh_init(shifter* s, int canonical, uint16_t K) {
    s->canonical = canonical; s->K = K;
    cyc_reset(&s->fw, K); cyc_reset(&s->rc, K);
}

typedef uint8_t (*base_fn)(const void* ctx, uint64_t i);

/* hash_base_impl (rollinghashshifter.hh:65-77, canonical :180-197) */
static void sh_hash_base(shifter* s, base_fn get, const void* ctx, uint64_t start) {
    cyc_reset(&s->fw, s->K); cyc_reset(&s->rc, s->K);
    for (uint16_t i = 0; i < s->K; ++i) {
        cyc_eat(&s->fw, get(ctx, start + i));
        if (s->canonical) cyc_eat(&s->rc, comp(get(ctx, start + s->K - 1 - i)));
    }
}
/* shift_right_impl (rollinghashshifter.hh:100-103, canonical :200-208) */
static inline void sh_shift_right(shifter* s, int out, int in) {
    cyc_update(&s->fw, out, in);
    if (s->canonical) cyc_reverse_update(&s->rc, comp(in), comp(out));
}
/* shift_left_impl (rollinghashshifter.hh:94-97, canonical :211-219) */
static inline void sh_shift_left(shifter* s, int in, int out) {
    cyc_reverse_update(&s->fw, in, out);
    if (s->canonical) cyc_update(&s->rc, comp(out), comp(in));
}
/* Hash::value / Canonical::value (canonical.hh:58-60, 124-126) */
static inline uint64_t sh_value(const shifter* s) {
    if (!s->canonical) return s->fw.h;
    return s->fw.h < s->rc.h ? s->fw.h : s->rc.h;
}

static uint8_t code_at(const void* ctx, uint64_t i) { return ((const uint8_t*)ctx)[i]; }
static uint8_t packed_at(const void* ctx, uint64_t i) {
    return (uint8_t)((((const uint32_t*)ctx)[i >> 4] >> ((i & 15u) << 1)) & 3u);
}

void orc_hash_codes(const uint8_t* codes, uint64_t len, uint16_t K,
                    uint64_t* fw, uint64_t* rc) {
    if (len < K) return;
    shifter s; sh_init(&s, 1, K);
    sh_hash_base(&s, code_at, codes, 0);
    fw[0] = s.fw.h; rc[0] = s.rc.h;
    for (uint64_t i = 1; i + K <= len; ++i) {
        sh_shift_right(&s, codes[i - 1], codes[i + K - 1]);
        fw[i] = s.fw.h; rc[i] = s.rc.h;
    }
}

/* ---- table sizing (storage.hh:146-190) -------------------------------- */

static int is_prime(uint64_t n) {
    if (n < 2) return 0;
    if (n == 2) return 1;
    if (n % 2 == 0) return 0;
    for (uint64_t i = 3; i * i <= n; i += 2)
        if (n % i == 0) return 0;
    return 1;
}

uint32_t orc_primes(uint32_t n, uint64_t x, uint64_t* out) {
    uint32_t got = 0;
    if (x == 1) { out[0] = 1; return 1; }
    uint64_t i = x - 1;
    if (i % 2 == 0) i--;
    while (got != n) {
        if (is_prime(i)) out[got++] = i;
        if (i == 1) break;
        i -= 2;
    }
    return got;
}

/* ---- storages ---------------------------------------------------------- */

struct orc_storage {
    int kind;
    int n;
    uint64_t sizes[64];
    uint8_t* t[64];
    uint64_t bytes[64];
    uint64_t n_unique, n_occupied;
};

orc_storage* orc_storage_new(int kind, const uint64_t* sizes, int n_tables) {
    if (n_tables < 1 || n_tables > 64) return NULL;
    orc_storage* s = (orc_storage*)calloc(1, sizeof(*s));
    s->kind = kind; s->n = n_tables;
    for (int i = 0; i < n_tables; ++i) {
        s->sizes[i] = sizes[i];
        /* BitStorage: size/8+1 (bitstorage.hh:143-156); ByteStorage: size
         * (bytestorage.hh:128-136); NibbleStorage: size/2+1 (nibblestorage.hh:166-177) */
        s->bytes[i] = kind == ORC_BIT ? sizes[i] / 8 + 1
                    : kind == ORC_NIBBLE ? sizes[i] / 2 + 1 : sizes[i];
        s->t[i] = (uint8_t*)calloc(s->bytes[i], 1);
    }
    return s;
}

void orc_storage_free(orc_storage* s) {
    if (!s) return;
    for (int i = 0; i < s->n; ++i) free(s->t[i]);
    free(s);
}

int orc_n_tables(const orc_storage* s) { return s->n; }
uint64_t orc_table_bytes(const orc_storage* s, int i) { return s->bytes[i]; }
const uint8_t* orc_table(const orc_storage* s, int i) { return s->t[i]; }
void orc_stats(const orc_storage* s, uint64_t* u, uint64_t* o) { *u = s->n_unique; *o = s->n_occupied; }

void orc_reset(orc_storage* s) {
    for (int i = 0; i < s->n; ++i) memset(s->t[i], 0, s->bytes[i]);
}

/* BitStorage::insert (bitstorage.hh:195-219) */
static int bit_insert(orc_storage* s, uint64_t h) {
    int is_new = 0;
    for (int i = 0; i < s->n; ++i) {
        uint64_t bin = h % s->sizes[i];
        uint8_t bit = (uint8_t)(1u << (bin % 8));
        uint8_t orig = s->t[i][bin / 8];
        s->t[i][bin / 8] = orig | bit;
        if (!(orig & bit)) {
            if (i == 0) s->n_occupied++;
            is_new = 1;
        }
    }
    if (is_new) s->n_unique++;
    return is_new;
}

/* ByteStorage::insert without bigcount (bytestorage.cc:60-113) */
static int byte_insert(orc_storage* s, uint64_t h) {
    int is_new = 0;
    for (int i = 0; i < s->n; ++i) {
        uint64_t bin = h % s->sizes[i];
        uint8_t cur = s->t[i][bin];
        if (!is_new && cur == 0) {
            is_new = 1;
            if (i == 0) s->n_occupied++;
        }
        if (cur < 255) s->t[i][bin] = (uint8_t)(cur + 1);
    }
    if (is_new) s->n_unique++;
    return is_new;
}

/* NibbleStorage layout: byte c/2, even c -> high nibble, odd -> low
 * (nibblestorage.hh:109-122); insert (nibblestorage.cc:60-100) */
static int nib_insert(orc_storage* s, uint64_t h) {
    int is_new = 0;
    for (int i = 0; i < s->n; ++i) {
        uint64_t c = h % s->sizes[i];
        uint64_t idx = c / 2;
        uint8_t mask = (c % 2) ? 0x0F : 0xF0;
        uint8_t shift = (c % 2) ? 0 : 4;
        uint8_t cur = (uint8_t)((s->t[i][idx] & mask) >> shift);
        if (!is_new && cur == 0) {
            is_new = 1;
            if (i == 0) s->n_occupied++;
        }
        if (cur == 15) continue;
        uint8_t nc = (uint8_t)((cur + 1) << shift);
        s->t[i][idx] = (uint8_t)((s->t[i][idx] & ~mask) | (nc & mask));
    }
    if (is_new) s->n_unique++;
    return is_new;
}

int orc_insert(orc_storage* s, uint64_t h) {
    switch (s->kind) {
    case ORC_BIT: return bit_insert(s, h);
    case ORC_BYTE: return byte_insert(s, h);
    default: return nib_insert(s, h);
    }
}

/* BitStorage::query (bitstorage.cc:87-100); ByteStorage::query
 * (bytestorage.cc:116-139); NibbleStorage::query (nibblestorage.cc:112-130) */
int16_t orc_query(const orc_storage* s, uint64_t h) {
    if (s->kind == ORC_BIT) {
        for (int i = 0; i < s->n; ++i) {
            uint64_t bin = h % s->sizes[i];
            if (!(s->t[i][bin / 8] & (1u << (bin % 8)))) return 0;
        }
        return 1;
    }
    if (s->kind == ORC_BYTE) {
        int16_t m = 255;
        for (int i = 0; i < s->n; ++i) {
            int16_t c = s->t[i][h % s->sizes[i]];
            if (c < m) m = c;
        }
        return m;
    }
    uint8_t m = 15;
    for (int i = 0; i < s->n; ++i) {
        uint64_t c = h % s->sizes[i];
        uint8_t v = (uint8_t)((s->t[i][c / 2] & ((c % 2) ? 0x0F : 0xF0)) >> ((c % 2) ? 0 : 4));
        if (v < m) m = v;
    }
    return m;
}

/* insert_and_query: Bit -> insert, 1 (bitstorage.cc:78-84); Byte/Nibble ->
 * 1 if new else query (bytestorage.cc:142-150, nibblestorage.cc:102-109) */
int16_t orc_insert_and_query(orc_storage* s, uint64_t h) {
    int is_new = orc_insert(s, h);
    if (s->kind == ORC_BIT) return 1;
    return is_new ? 1 : orc_query(s, h);
}

/* ---- dBG over read batches (dbg.hh:249-394, kmeriterator.hh:63-123) ---- */

uint64_t orc_count_kmers(uint16_t K, const uint64_t* off, uint64_t n) {
    uint64_t t = 0;
    for (uint64_t r = 0; r < n; ++r) {
        uint64_t L = off[r + 1] - off[r];
        if (L >= K) t += L - K + 1;
    }
    return t;
}

typedef void (*kmer_cb)(void* ctx, uint64_t read, uint64_t pos, const shifter* s);

/* KmerIterator: hash_base over the first K bases, then
 * shift_right(seq[i-1], seq[i+K-1]) per step (kmeriterator.hh:63-123).
 * Reads shorter than K raise SequenceLengthException in the reference
 * (kmeriterator.hh:72-74); here they are skipped, as InserterProcessor does. */
static void walk_reads(int canonical, uint16_t K, const uint32_t* packed,
                       const uint64_t* off, uint64_t n, uint64_t r0, uint64_t stride,
                       kmer_cb cb, void* ctx) {
    shifter s; sh_init(&s, canonical, K);
    for (uint64_t r = r0; r < n; r += stride) {
        uint64_t b = off[r], L = off[r + 1] - off[r];
        if (L < K) continue;
        sh_hash_base(&s, packed_at, packed, b);
        cb(ctx, r, 0, &s);
        for (uint64_t i = 1; i + K <= L; ++i) {
            sh_shift_right(&s, packed_at(packed, b + i - 1), packed_at(packed, b + i + K - 1));
            cb(ctx, r, i, &s);
        }
    }
}

typedef struct { uint64_t* val; uint64_t* fw; uint64_t* rc; uint64_t k; } hash_ctx;
static void hash_cb(void* c, uint64_t r, uint64_t p, const shifter* s) {
    (void)r; (void)p;   /* the read walker's callback signature */
    hash_ctx* h = (hash_ctx*)c;
    if (h->val) h->val[h->k] = sh_value(s);
    if (h->fw) h->fw[h->k] = s->fw.h;
    if (h->rc) h->rc[h->k] = s->canonical ? s->rc.h : 0;
    h->k++;
}

void orc_hash_reads(int canonical, uint16_t K, const uint32_t* packed,
                    const uint64_t* off, uint64_t n, uint64_t* val, uint64_t* fw, uint64_t* rc) {
    hash_ctx h = {val, fw, rc, 0};
    walk_reads(canonical, K, packed, off, n, 0, 1, hash_cb, &h);
}

typedef struct { orc_storage* s; uint64_t* n_new; uint64_t total; } ins_ctx;
static void ins_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    ins_ctx* x = (ins_ctx*)c;
    int nw = orc_insert(x->s, sh_value(sh));
    if (x->n_new) x->n_new[r] += (uint64_t)nw;
    x->total++;
}

/* dBG::insert_sequence(seq, n_new) per read in batch order (dbg.hh:296-305) */
uint64_t orc_insert_reads(orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                          const uint64_t* off, uint64_t n, uint64_t* n_new) {
    if (n_new) memset(n_new, 0, n * sizeof(uint64_t));
    ins_ctx x = {s, n_new, 0};
    walk_reads(canonical, K, packed, off, n, 0, 1, ins_cb, &x);
    return x.total;
}

typedef struct { orc_storage* s; int16_t* counts; uint64_t k; } iq_ctx;
static void iq_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    iq_ctx* x = (iq_ctx*)c;
    x->counts[x->k++] = orc_insert_and_query(x->s, sh_value(sh));
}

/* dBG::insert_and_query_sequence (dbg.hh:327-340) */
void orc_insert_and_query_reads(orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                                const uint64_t* off, uint64_t n, int16_t* counts) {
    iq_ctx x = {s, counts, 0};
    walk_reads(canonical, K, packed, off, n, 0, 1, iq_cb, &x);
}

typedef struct { const orc_storage* s; int16_t* counts; uint64_t k; } q_ctx;
static void q_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    q_ctx* x = (q_ctx*)c;
    x->counts[x->k++] = orc_query(x->s, sh_value(sh));
}

/* dBG::query_sequence (dbg.hh:349-362) */
void orc_query_reads(const orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                     const uint64_t* off, uint64_t n, int16_t* counts) {
    q_ctx x = {s, counts, 0};
    walk_reads(canonical, K, packed, off, n, 0, 1, q_cb, &x);
}

/* Neighbour mask per k-mer: the cursor is the current k-mer;
 * left_extensions = for sym in "ACGT": shift_left(sym, back), record,
 * shift_right(sym, back) (hashextender.hh:352-364); right_extensions =
 * shift_right(front, sym), record, shift_left(front, sym) (:386-396); a
 * neighbour is present when query() != 0 (unitig_walker.hh:361-372).
 * bit i = left "ACGT"[i], bit 4+i = right "ACGT"[i]. */
typedef struct { const orc_storage* s; uint8_t* masks; uint64_t k;
                 const uint32_t* packed; const uint64_t* off; uint16_t K; } m_ctx;
static void m_cb(void* c, uint64_t r, uint64_t p, const shifter* cur) {
    m_ctx* x = (m_ctx*)c;
    uint64_t b = x->off[r] + p;
    int front = packed_at(x->packed, b), back = packed_at(x->packed, b + x->K - 1);
    shifter s = *cur;
    uint8_t m = 0;
    for (int sym = 0; sym < 4; ++sym) {
        sh_shift_left(&s, sym, back);
        if (orc_query(x->s, sh_value(&s))) m |= (uint8_t)(1u << sym);
        sh_shift_right(&s, sym, back);
    }
    for (int sym = 0; sym < 4; ++sym) {
        sh_shift_right(&s, front, sym);
        if (orc_query(x->s, sh_value(&s))) m |= (uint8_t)(1u << (4 + sym));
        sh_shift_left(&s, front, sym);
    }
    x->masks[x->k++] = m;
}

void orc_decision_masks(const orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                        const uint64_t* off, uint64_t n, uint8_t* masks) {
    m_ctx x = {s, masks, 0, packed, off, K};
    walk_reads(canonical, K, packed, off, n, 0, 1, m_cb, &x);
}

/* ---- compactor query (compactor.hh:346-466) ------------------------------ */
/* Per k-mer of a read, against the storage as it is: flags bit 0 = new
 * (query() == 0), bit 1 = seen (the hash is already in the read's new-k-mer
 * set at this position); mask = neighbour mask where a neighbour is present
 * when query() != 0 or it is one of the read's new k-mers (filter_nodes with
 * extras, unitig_walker.hh:457-469). */
typedef struct { uint64_t h; uint64_t p; } hp_pair;
static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}
static int cmp_hp(const void* a, const void* b) {
    const hp_pair* x = (const hp_pair*)a; const hp_pair* y = (const hp_pair*)b;
    if (x->h != y->h) return x->h < y->h ? -1 : 1;
    return x->p < y->p ? -1 : x->p > y->p;
}
typedef struct { uint64_t* h; uint64_t k; } collect_ctx;
static void collect_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    collect_ctx* x = (collect_ctx*)c;
    x->h[x->k++] = sh_value(sh);
}
typedef struct {
    const orc_storage* s; const uint64_t* set; uint64_t n_set;
    uint8_t* masks; uint64_t k; const uint32_t* packed; const uint64_t* off; uint16_t K;
} cm_ctx;
static int in_set(const cm_ctx* x, uint64_t h) {
    return x->n_set && bsearch(&h, x->set, x->n_set, sizeof(uint64_t), cmp_u64) != NULL;
}
static void cm_cb(void* c, uint64_t r, uint64_t p, const shifter* cur) {
    cm_ctx* x = (cm_ctx*)c;
    uint64_t b = x->off[r] + p;
    int front = packed_at(x->packed, b), back = packed_at(x->packed, b + x->K - 1);
    shifter s = *cur;
    uint8_t m = 0;
    for (int sym = 0; sym < 4; ++sym) {
        sh_shift_left(&s, sym, back);
        uint64_t h = sh_value(&s);
        if (orc_query(x->s, h) || in_set(x, h)) m |= (uint8_t)(1u << sym);
        sh_shift_right(&s, sym, back);
    }
    for (int sym = 0; sym < 4; ++sym) {
        sh_shift_right(&s, front, sym);
        uint64_t h = sh_value(&s);
        if (orc_query(x->s, h) || in_set(x, h)) m |= (uint8_t)(1u << (4 + sym));
        sh_shift_left(&s, front, sym);
    }
    x->masks[x->k++] = m;
}

void orc_compactor_reads(const orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                         const uint64_t* off, uint64_t n, uint8_t* flags, uint8_t* masks) {
    uint64_t k0 = 0;
    for (uint64_t r = 0; r < n; ++r) {
        uint64_t L = off[r + 1] - off[r];
        if (L < K) continue;
        uint64_t nk = L - K + 1;
        uint64_t* h = (uint64_t*)malloc(nk * sizeof(uint64_t));
        hp_pair* pairs = (hp_pair*)malloc(nk * sizeof(hp_pair));
        uint64_t* set = (uint64_t*)malloc(nk * sizeof(uint64_t));
        collect_ctx cc = {h, 0};
        walk_reads(canonical, K, packed, off + r, 1, 0, 1, collect_cb, &cc);
        uint64_t np = 0;
        for (uint64_t p = 0; p < nk; ++p) {
            int is_new = orc_query(s, h[p]) == 0;
            flags[k0 + p] = (uint8_t)is_new;
            if (is_new) { pairs[np].h = h[p]; pairs[np].p = p; ++np; }
        }
        qsort(pairs, np, sizeof(hp_pair), cmp_hp);
        uint64_t ns = 0;
        for (uint64_t i = 0; i < np; ++i) {
            if (i > 0 && pairs[i].h == pairs[i - 1].h) flags[k0 + pairs[i].p] |= 2;   /* seen */
            else set[ns++] = pairs[i].h;
        }
        cm_ctx mc = {s, set, ns, masks + k0, 0, packed, off + r, K};
        /* walk_reads indexes offsets by the local read 0 */
        walk_reads(canonical, K, packed, off + r, 1, 0, 1, cm_cb, &mc);
        free(h); free(pairs); free(set);
        k0 += nk;
    }
}

/* ---- multi-threaded insert (throughput baseline) ----------------------- */
/* Atomic cell updates in the spirit of the reference's thread-safe storages
 * (__sync_fetch_and_or bitstorage.hh:203-209; __sync_add_and_fetch
 * bytestorage.cc:89).  Saturation uses compare-and-swap so final bytes stay
 * exact. */
static void atomic_insert(orc_storage* s, uint64_t h) {
    for (int i = 0; i < s->n; ++i) {
        uint64_t c = h % s->sizes[i];
        if (s->kind == ORC_BIT) {
            __atomic_fetch_or(&s->t[i][c / 8], (uint8_t)(1u << (c % 8)), __ATOMIC_RELAXED);
        } else if (s->kind == ORC_BYTE) {
            uint8_t* p = &s->t[i][c];
            uint8_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
            while (cur < 255 && !__atomic_compare_exchange_n(p, &cur, (uint8_t)(cur + 1), 1,
                                                             __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {}
        } else {
            uint8_t* p = &s->t[i][c / 2];
            unsigned sh = (c % 2) ? 0 : 4;
            uint8_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
            while (((cur >> sh) & 15u) < 15u &&
                   !__atomic_compare_exchange_n(p, &cur, (uint8_t)(cur + (1u << sh)), 1,
                                                __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {}
        }
    }
}

typedef struct { orc_storage* s; uint64_t total; } mt_ctx;
static void mt_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    mt_ctx* x = (mt_ctx*)c;
    atomic_insert(x->s, sh_value(sh));
    x->total++;
}

typedef struct {
    orc_storage* s; int canonical; uint16_t K; const uint32_t* packed;
    const uint64_t* off; uint64_t n; uint64_t r0, stride; uint64_t total;
} mt_job;

static void* mt_run(void* arg) {
    mt_job* j = (mt_job*)arg;
    mt_ctx x = {j->s, 0};
    walk_reads(j->canonical, j->K, j->packed, j->off, j->n, j->r0, j->stride, mt_cb, &x);
    j->total = x.total;
    return NULL;
}

uint64_t orc_insert_reads_mt(orc_storage* s, int canonical, uint16_t K, const uint32_t* packed,
                             const uint64_t* off, uint64_t n, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    mt_job* jobs = (mt_job*)calloc((size_t)n_threads, sizeof(mt_job));
    for (int t = 0; t < n_threads; ++t) {
        mt_job j = {s, canonical, K, packed, off, n, (uint64_t)t, (uint64_t)n_threads, 0};
        jobs[t] = j;
        pthread_create(&th[t], NULL, mt_run, &jobs[t]);
    }
    uint64_t total = 0;
    for (int t = 0; t < n_threads; ++t) { pthread_join(th[t], NULL); total += jobs[t].total; }
    free(th); free(jobs);
    return total;
}

/* ---- touch counts of a cell range (the final-state check of long runs) --
 * The final value of a cell of a saturating table is min(max, the number of
 * k-mer inserts that hit it), whatever their order (bytestorage.cc:60-113,
 * nibblestorage.cc:60-100 each add one up to the maximum).  This counts, for
 * the tables listed in `tables`, the inserts that hit cells [lo[j],
 * lo[j] + width) -- min(255, count) per cell into out[j * width + cell - lo[j]]
 * -- over every k-mer of the batch, on n_threads threads. */
typedef struct {
    const uint64_t* sizes; const int* tables; int n_sel; const uint64_t* lo; uint64_t width;
    uint8_t* cnt;
} cc_ctx;
static void cc_cb(void* c, uint64_t r, uint64_t p, const shifter* sh) {
    (void)r; (void)p;   /* the read walker's callback signature */
    cc_ctx* x = (cc_ctx*)c;
    const uint64_t h = sh_value(sh);
    for (int j = 0; j < x->n_sel; ++j) {
        const uint64_t cell = h % x->sizes[x->tables[j]];
        if (cell >= x->lo[j] && cell - x->lo[j] < x->width) {
            uint8_t* q = &x->cnt[(uint64_t)j * x->width + (cell - x->lo[j])];
            if (*q < 255) ++*q;
        }
    }
}
typedef struct {
    cc_ctx c; int canonical; uint16_t K; const uint32_t* packed; const uint64_t* off;
    uint64_t n, r0, stride;
} cc_job;
/* The same walk as walk_reads + cc_cb (hash_base, then shift_right per
 * step), with the base reads and the roll inlined: this check hashes every
 * k-mer of a multi-gigabase stream. */
static void* cc_run(void* arg) {
    cc_job* j = (cc_job*)arg;
    const uint16_t K = j->K;
    const unsigned myr = K % 64u;
    uint64_t outw[4];
    for (int c = 0; c < 4; ++c) outw[c] = rotl64(SYM[c], myr);
    const uint32_t* pk = j->packed;
    for (uint64_t r = j->r0; r < j->n; r += j->stride) {
        const uint64_t b = j->off[r], L = j->off[r + 1] - j->off[r];
        if (L < K) continue;
        uint64_t fw = 0, rc = 0;
        for (uint16_t i = 0; i < K; ++i) {
            const unsigned c = (pk[(b + i) >> 4] >> (((b + i) & 15u) << 1)) & 3u;
            fw = rotl64(fw, 1) ^ SYM[c];
            const unsigned d = (pk[(b + K - 1 - i) >> 4] >> (((b + K - 1 - i) & 15u) << 1)) & 3u;
            rc = rotl64(rc, 1) ^ SYM[comp((int)d)];
        }
        for (uint64_t i = 0;; ++i) {
            shifter s;   /* value() of the current k-mer, as sh_value */
            s.canonical = j->canonical; s.fw.h = fw; s.rc.h = rc;
            cc_cb(&j->c, r, i, &s);
            if (i + K >= L) break;
            const unsigned out = (pk[(b + i) >> 4] >> (((b + i) & 15u) << 1)) & 3u;
            const unsigned in = (pk[(b + i + K) >> 4] >> (((b + i + K) & 15u) << 1)) & 3u;
            fw = rotl64(fw, 1) ^ outw[out] ^ SYM[in];                       /* update */
            const uint64_t x = rc ^ outw[comp((int)in)] ^ SYM[comp((int)out)]; /* reverse_update */
            rc = (x >> 1) | (x << 63);
        }
    }
    return NULL;
}

int orc_count_cells(int canonical, uint16_t K, const uint32_t* packed, const uint64_t* off,
                    uint64_t n, const uint64_t* sizes, const int* tables, int n_sel,
                    const uint64_t* lo, uint64_t width, uint8_t* out, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_sel < 1 || width == 0) return 1;
    const uint64_t cells = (uint64_t)n_sel * width;
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    cc_job* jobs = (cc_job*)calloc((size_t)n_threads, sizeof(cc_job));
    int ok = th && jobs;
    for (int t = 0; ok && t < n_threads; ++t) {
        uint8_t* cnt = (uint8_t*)calloc(cells, 1);
        cc_job j = {{sizes, tables, n_sel, lo, width, cnt}, canonical, K, packed, off, n,
                    (uint64_t)t, (uint64_t)n_threads};
        jobs[t] = j;
        ok = cnt != NULL;
    }
    if (!ok) {   /* nothing started: free what was allocated */
        for (int t = 0; jobs && t < n_threads; ++t) free(jobs[t].c.cnt);
        free(th); free(jobs);
        return 2;
    }
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, cc_run, &jobs[t]);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    for (uint64_t i = 0; i < cells; ++i) {
        unsigned v = out[i];
        for (int t = 0; t < n_threads && v < 255; ++t) v += jobs[t].c.cnt[i];
        out[i] = (uint8_t)(v < 255 ? v : 255);
    }
    for (int t = 0; t < n_threads; ++t) free(jobs[t].c.cnt);
    free(th); free(jobs);
    return 0;
}

/* ---- FASTX parser policy (readers.hh:150-219, alphabets.hh:41-56,107-130) */

int64_t orc_pack_ascii(const char* seqs, const uint64_t* so, uint64_t n, uint32_t min_length,
                       uint32_t* packed, uint64_t* off, uint64_t* n_skipped) {
    uint64_t kept = 0, pos = 0, skipped = 0;
    off[0] = 0;
    for (uint64_t r = 0; r < n; ++r) {
        const char* s = seqs + so[r];
        uint64_t L = so[r + 1] - so[r];
        int ok = 1;
        for (uint64_t i = 0; i < L && ok; ++i) {
            char c = s[i];
            ok = c == 'A' || c == 'C' || c == 'G' || c == 'T' ||
                 c == 'a' || c == 'c' || c == 'g' || c == 't';
        }
        if (!ok || L < min_length) { skipped++; continue; }
        for (uint64_t i = 0; i < L; ++i) {
            char c = s[i];
            uint32_t code = (c == 'A' || c == 'a') ? 0 : (c == 'C' || c == 'c') ? 1
                          : (c == 'G' || c == 'g') ? 2 : 3;
            uint64_t j = pos + i;
            if ((j & 15u) == 0) packed[j >> 4] = 0;
            packed[j >> 4] |= code << ((j & 15u) << 1);
        }
        pos += L;
        off[++kept] = pos;
    }
    *n_skipped = skipped;
    return (int64_t)kept;
}

/* ---- FASTA/FASTQ records (kseq.h:88-220, readers.hh:150-219) ------------ */

/* The stream: text[pos..n).  ks_getc (kseq.h: one byte, -1 at the end). */
typedef struct {
    const char* s;
    uint64_t n, pos;
} orc_ks;

static int ks_getc_(orc_ks* k) { return k->pos < k->n ? (unsigned char)k->s[k->pos++] : -1; }

/* kstring_t (kseq.h:78-82): a growing byte string. */
typedef struct {
    char* s;
    uint64_t l, cap;
} orc_kstr;

static void kstr_put(orc_kstr* t, const char* src, uint64_t m) {
    if (t->l + m + 1 > t->cap) {
        t->cap = 2 * (t->l + m) + 64;
        t->s = (char*)realloc(t->s, t->cap);
    }
    memcpy(t->s + t->l, src, m);
    t->l += m;
}

static int ks_isspace(int c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

/* ks_getuntil2 (kseq.h:88-139) with KS_SEP_SPACE (line = 0) or KS_SEP_LINE
 * (line = 1): bytes up to the delimiter go to t (appended when append), the
 * delimiter is consumed and reported in *dret (0 at the end of the text).
 * -1 when the text had ended before the call; else the string's length,
 * after dropping one trailing '\r' of a line string longer than one byte. */
static int64_t ks_until(orc_ks* k, int line, orc_kstr* t, int append, int* dret) {
    if (dret) *dret = 0;
    if (!append) t->l = 0;
    if (k->pos >= k->n) return -1;
    uint64_t i = k->pos;
    while (i < k->n && !(line ? k->s[i] == '\n' : ks_isspace((unsigned char)k->s[i]))) ++i;
    kstr_put(t, k->s + k->pos, i - k->pos);
    if (i < k->n && dret) *dret = (unsigned char)k->s[i];
    k->pos = i < k->n ? i + 1 : k->n;
    if (line && t->l > 1 && t->s[t->l - 1] == '\r') --t->l;
    return (int64_t)t->l;
}

/* kseq_read (kseq.h:173-220): >= 0 the sequence length, -1 end, -2 the
 * sequence and quality lengths differ (or no quality line). */
static int64_t kseq_read_(orc_ks* k, int* last_char, orc_kstr* name, orc_kstr* comment,
                          orc_kstr* seq, orc_kstr* qual) {
    int c;
    if (*last_char == 0) {
        while ((c = ks_getc_(k)) >= 0 && c != '>' && c != '@') {}
        if (c < 0) return c;
        *last_char = c;
    }
    comment->l = seq->l = qual->l = 0;
    const int64_t r = ks_until(k, 0, name, 0, &c);
    if (r < 0) return r;
    if (c != '\n') ks_until(k, 1, comment, 0, NULL);
    while ((c = ks_getc_(k)) >= 0 && c != '>' && c != '+' && c != '@') {
        if (c == '\n') continue;   /* empty lines */
        const char ch = (char)c;
        kstr_put(seq, &ch, 1);
        ks_until(k, 1, seq, 1, NULL);
    }
    if (c == '>' || c == '@') *last_char = c;
    if (c != '+') return (int64_t)seq->l;   /* FASTA */
    while ((c = ks_getc_(k)) >= 0 && c != '\n') {}   /* rest of the '+' line */
    if (c == -1) return -2;
    while (ks_until(k, 1, qual, 1, NULL) >= 0 && qual->l < seq->l) {}
    *last_char = 0;
    if (seq->l != qual->l) return -2;
    return (int64_t)seq->l;
}

int64_t orc_parse_fastx(const char* text, uint64_t n, uint32_t min_length, char* seq_out,
                        uint64_t seq_cap, uint64_t* seq_off, uint64_t rec_cap,
                        uint64_t stats[4]) {
    orc_ks k = {text, n, 0};
    int last_char = 0;
    orc_kstr name = {0}, comment = {0}, seq = {0}, qual = {0};
    uint64_t kept = 0, used = 0;
    int64_t ret = 0;
    stats[0] = stats[1] = stats[2] = stats[3] = 0;
    seq_off[0] = 0;
    for (;;) {
        const int64_t stat = kseq_read_(&k, &last_char, &name, &comment, &seq, &qual);
        if (stat == -1) break;
        if (stat == -2) {
            stats[1]++;
            stats[3] = stats[0];
            ret = -2;
            break;
        }
        /* FastxParser::next: Alphabet::validate, then the length filter */
        int valid = 1;
        for (uint64_t i = 0; i < seq.l; ++i) {
            const char c = seq.s[i];
            const char u = (c == 'a') ? 'A' : (c == 'c') ? 'C' : (c == 'g') ? 'G' : (c == 't') ? 'T' : c;
            if (u != 'A' && u != 'C' && u != 'G' && u != 'T') { valid = 0; break; }
            seq.s[i] = u;
        }
        int keep = valid;
        if (!valid) stats[1]++;
        if (seq.l < min_length) { keep = 0; stats[1]++; }
        stats[0]++;
        if (!keep) { stats[2]++; continue; }
        if (kept >= rec_cap || used + seq.l > seq_cap) { ret = -5; break; }
        memcpy(seq_out + used, seq.s, seq.l);
        used += seq.l;
        seq_off[++kept] = used;
    }
    free(name.s); free(comment.s); free(seq.s); free(qual.s);
    return ret < 0 ? ret : (int64_t)kept;
}
