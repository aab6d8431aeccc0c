// Device-side building blocks for the GB300 dBG hot path: the cyclic rolling
// hash on 2-bit codes, exact 64-bit modulo by the table primes, cell
// addressing for the three storages, and the per-window first-touch claims map.
//
// Reference semantics (goetia, paths relative to its source tree):
//   CyclicHash eat/update/reverse_update  include/goetia/hashing/rollinghash/cyclichash.h:85-108
//   Canonical shifter                     include/goetia/hashing/rollinghashshifter.hh:180-219
//   BitStorage / ByteStorage / NibbleStorage cell layout
//       bitstorage.hh:195-219, bytestorage.cc:60-113, nibblestorage.hh:109-122
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gdbg_types.h"

namespace gdbg {

// CharacterHash::hashvalues for 'A','C','G','T' (characterhash.h:49-56,
// Lemire rollinghashcpp, Apache-2.0).  A hash depends on these exact words.
constexpr uint64_t SYM_A = 16664410744025174816ull;
constexpr uint64_t SYM_C = 15956807086001210932ull;
constexpr uint64_t SYM_G = 9404339731978646439ull;
constexpr uint64_t SYM_T = 836480985777824379ull;

__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x << r) | (x >> (64u - r)) : x;
}
__host__ __device__ __forceinline__ uint64_t rotl1(uint64_t x) { return (x << 1) | (x >> 63); }
__host__ __device__ __forceinline__ uint64_t rotr1(uint64_t x) { return (x >> 1) | (x << 63); }

// Host side: the kernels' hash constants for K, the four symbol words rotated
// by K mod 64 (the term CyclicHash::update removes, cyclichash.h:85-92).
inline HashParams make_hash_params(uint32_t K) {
    const uint64_t words[4] = {SYM_A, SYM_C, SYM_G, SYM_T};
    HashParams hp{};
    hp.K = K;
    for (int c = 0; c < 4; ++c) hp.tk[c] = rotl64(words[c], K % 64u);
    return hp;
}

// Symbol word for a 2-bit code, selected in registers (no indexed memory).
__device__ __forceinline__ uint64_t sym(uint32_t c) {
    uint64_t lo = (c & 1u) ? SYM_C : SYM_A;
    uint64_t hi = (c & 1u) ? SYM_T : SYM_G;
    return (c & 2u) ? hi : lo;
}
// Same for the rotated-by-K copies held in `tk` (4 words, kernel params).
__device__ __forceinline__ uint64_t symk(const HashParams& hp, uint32_t c) {
    uint64_t lo = (c & 1u) ? hp.tk[1] : hp.tk[0];
    uint64_t hi = (c & 1u) ? hp.tk[3] : hp.tk[2];
    return (c & 2u) ? hi : lo;
}

// Exact h % p with a precomputed m = floor((2^64-1)/p).  q = mulhi(h, m) is
// never above floor(h/p) and at most one below it, so a single conditional
// subtraction finishes the reduction (Barrett, one correction step).
__device__ __forceinline__ uint64_t fastmod(uint64_t h, uint64_t p, uint64_t m) {
    uint64_t q = __umul64hi(h, m);
    uint64_t r = h - q * p;
    return r >= p ? r - p : r;
}
// fastmod for p < 2^31.  The Barrett quotient is floor(h/p) or one less, so
// the remainder before the correction is below 2p <= 2^32 and its low 32
// bits are exact: one 32-bit multiply-subtract and an unsigned min.
__device__ __forceinline__ uint32_t fastmod_small(uint64_t h, uint32_t p, uint64_t m) {
    const uint64_t q = __umul64hi(h, m);
    const uint32_t r = (uint32_t)h - (uint32_t)q * p;
    return min(r, r - p);
}

// ---- 2-bit packed base stream ---------------------------------------------
// base j lives in bits 2*(j%16) of word j/16.
__device__ __forceinline__ uint32_t base_at(const uint32_t* __restrict__ packed, uint64_t j) {
    return (__ldg(packed + (j >> 4)) >> ((uint32_t)(j & 15u) << 1)) & 3u;
}

// Sequential reader that loads each packed word once, and only when a base
// of that word is consumed (so it never reads past the last base it returns).
struct BaseCursor {
    const uint32_t* __restrict__ packed;
    uint64_t pos;
    uint32_t word;
    bool loaded;
    __device__ __forceinline__ void init(const uint32_t* p, uint64_t j) {
        packed = p; pos = j; loaded = false;
    }
    __device__ __forceinline__ uint32_t next() {
        if (!loaded || (pos & 15u) == 0) {
            word = __ldg(packed + (pos >> 4)) >> ((uint32_t)(pos & 15u) << 1);
            loaded = true;
        }
        uint32_t c = word & 3u;
        ++pos;
        word >>= 2;
        return c;
    }
};

// Seed the hash of the k-mer whose first base is at `b`:
//   fw = XOR_i rotl(T[s_i], K-1-i)              (K eats, cyclichash.h:105-108)
//   rc = XOR_m rotl(T[comp(s_m)], m)            (eats of the reverse complement,
//                                                rollinghashshifter.hh:180-197)
template <bool CANON>
__device__ __forceinline__ void seed_hash(const uint32_t* __restrict__ packed, uint64_t b,
                                          uint32_t K, uint64_t& fw, uint64_t& rc) {
    BaseCursor cur;
    cur.init(packed, b);
    fw = 0; rc = 0;
    for (uint32_t i = 0; i < K; ++i) {
        uint32_t c = cur.next();
        fw = rotl1(fw) ^ sym(c);
        if (CANON) rc ^= rotl64(sym(3u - c), i);
    }
}

// Roll one base to the right: drop `out`, append `in`
//   fw: update(out, in)                           (cyclichash.h:85-92)
//   rc: reverse_update(comp(in), comp(out))       (rollinghashshifter.hh:200-208)
template <bool CANON>
__device__ __forceinline__ void roll_right(const HashParams& hp, uint32_t out, uint32_t in,
                                           uint64_t& fw, uint64_t& rc) {
    fw = rotl1(fw) ^ symk(hp, out) ^ sym(in);
    if (CANON) rc = rotr1(rc ^ symk(hp, 3u - in) ^ sym(3u - out));
}
// Roll one base to the left: prepend `in`, drop `out` (shift_left_impl,
// rollinghashshifter.hh:211-219)
template <bool CANON>
__device__ __forceinline__ void roll_left(const HashParams& hp, uint32_t in, uint32_t out,
                                          uint64_t& fw, uint64_t& rc) {
    fw = rotr1(fw ^ symk(hp, in) ^ sym(out));
    if (CANON) rc = rotl1(rc) ^ symk(hp, 3u - out) ^ sym(3u - in);
}

template <bool CANON>
__device__ __forceinline__ uint64_t hash_value(uint64_t fw, uint64_t rc) {
    if (!CANON) return fw;
    return fw < rc ? fw : rc;   // Canonical::value (canonical.hh:124-126)
}

// ---- storage cells -----------------------------------------------------
// Tables are stored as 32-bit words; byte b of the reference's byte array is
// byte b%4 of word b/4 (little endian), so word contents equal the
// reference's bytes when copied out.
struct Cell {
    uint32_t* word;
    uint32_t shift;  // bit offset of the cell inside the word
};

template <int STORAGE>
__device__ __forceinline__ Cell cell_of(const TableParams& tp, int i, uint64_t bin) {
    Cell c;
    uint32_t* base = tp.words[i];
    if (STORAGE == GDBG_BIT) {            // byte bin/8, bit bin%8
        c.word = base + (bin >> 5);
        c.shift = (uint32_t)(bin & 31u);
    } else if (STORAGE == GDBG_BYTE) {    // byte bin
        c.word = base + (bin >> 2);
        c.shift = (uint32_t)(bin & 3u) << 3;
    } else {                              // byte bin/2; even bin -> high nibble
        uint64_t byte = bin >> 1;
        c.word = base + (byte >> 2);
        c.shift = ((uint32_t)(byte & 3u) << 3) + ((bin & 1u) ? 0u : 4u);
    }
    return c;
}

template <int STORAGE>
__device__ __forceinline__ uint32_t cell_value(uint32_t word, uint32_t shift) {
    if (STORAGE == GDBG_BIT) return (word >> shift) & 1u;
    if (STORAGE == GDBG_BYTE) return (word >> shift) & 0xFFu;
    return (word >> shift) & 0xFu;
}

// Region-relative cell address in shared memory words.
template <int STORAGE>
__device__ __forceinline__ void region_cell(uint32_t co, uint32_t& word, uint32_t& shift) {
    if (STORAGE == GDBG_BIT) {
        word = co >> 5;
        shift = co & 31u;
    } else if (STORAGE == GDBG_BYTE) {
        word = co >> 2;
        shift = (co & 3u) << 3;
    } else {
        const uint32_t byte = co >> 1;
        word = byte >> 2;
        shift = ((byte & 3u) << 3) + ((co & 1u) ? 0u : 4u);
    }
}

template <int STORAGE>
__host__ __device__ constexpr uint32_t cells_per_word() {
    return STORAGE == GDBG_BIT ? 32u : STORAGE == GDBG_BYTE ? 4u : 8u;
}

template <int STORAGE>
__device__ __forceinline__ uint32_t cell_max() {
    return STORAGE == GDBG_BIT ? 1u : STORAGE == GDBG_BYTE ? 255u : 15u;
}

// Saturating increment of one cell by compare-and-swap on its word, starting
// from a guess of the word's contents.  Final contents are
// min(max, start + touches) whatever the order, which is what the
// reference's sequential loop produces.
template <int STORAGE>
__device__ __forceinline__ bool sat_increment(uint32_t* word, uint32_t shift, uint32_t guess,
                                              uint32_t* err) {
    uint32_t cur = guess;
    for (int it = 0; it < (1 << 20); ++it) {
        if (cell_value<STORAGE>(cur, shift) >= cell_max<STORAGE>()) return true;
        uint32_t prev = atomicCAS(word, cur, cur + (1u << shift));
        if (prev == cur) return true;
        cur = prev;
    }
    atomicOr(err, GDBG_ERR_CAS_LIMIT);
    return false;
}

// ---- first-touch claims --------------------------------------------------
// Open-addressing map from cell id (table << 32 | cell) to the smallest
// window-local k-mer ordinal that touched the cell while it was zero at the
// window start.  One 64-bit slot: epoch (7) | ordinal (20) | cell id (37).
// Slots from another epoch count as empty, so the map is only cleared when
// the 7-bit epoch wraps.
constexpr int CLAIM_EPOCH_BITS = 7;
constexpr int CLAIM_ORD_BITS = 20;
constexpr int CLAIM_ID_BITS = 37;
constexpr uint64_t CLAIM_ID_MASK = (1ull << CLAIM_ID_BITS) - 1;
constexpr uint64_t CLAIM_ORD_MASK = (1ull << CLAIM_ORD_BITS) - 1;

__device__ __forceinline__ uint32_t claim_epoch(uint64_t s) { return (uint32_t)(s >> 57); }
__device__ __forceinline__ uint32_t claim_ord(uint64_t s) { return (uint32_t)((s >> 37) & CLAIM_ORD_MASK); }
__device__ __forceinline__ uint64_t claim_id(uint64_t s) { return s & CLAIM_ID_MASK; }
__device__ __forceinline__ uint64_t claim_pack(uint32_t epoch, uint32_t ord, uint64_t id) {
    return ((uint64_t)epoch << 57) | ((uint64_t)ord << 37) | id;
}
__device__ __forceinline__ uint32_t claim_slot(uint64_t id, uint32_t mask) {
    uint64_t x = id * 0x9E3779B97F4A7C15ull;
    return (uint32_t)(x >> 32) & mask;
}

// Record `ord` for cell `id`, keeping the minimum.  Returns true when this
// call created the entry (the cell's first claim in this epoch).
__device__ __forceinline__ bool claim_min(uint64_t* __restrict__ map, uint32_t mask,
                                          uint32_t epoch, uint64_t id, uint32_t ord,
                                          uint32_t* err) {
    uint32_t s = claim_slot(id, mask);
    uint64_t want = claim_pack(epoch, ord, id);
    uint64_t cur = *(volatile uint64_t*)(map + s);
    for (uint32_t it = 0; it <= mask; ) {
        if (claim_epoch(cur) != epoch) {
            uint64_t prev = atomicCAS((unsigned long long*)(map + s), cur, want);
            if (prev == cur) return true;
            cur = prev;
            continue;
        }
        if (claim_id(cur) == id) {
            if (claim_ord(cur) <= ord) return false;
            uint64_t prev = atomicCAS((unsigned long long*)(map + s), cur, want);
            if (prev == cur) return false;
            cur = prev;
            continue;
        }
        s = (s + 1) & mask;
        ++it;
        cur = *(volatile uint64_t*)(map + s);
    }
    atomicOr(err, GDBG_ERR_CLAIMS_FULL);
    return false;
}

// Smallest ordinal recorded for `id` in this epoch (0xFFFFFFFF when absent,
// which only happens after a reported error).
__device__ __forceinline__ uint32_t claim_lookup(const uint64_t* __restrict__ map, uint32_t mask,
                                                 uint32_t epoch, uint64_t id) {
    uint32_t s = claim_slot(id, mask);
    for (uint32_t it = 0; it <= mask; ++it) {
        uint64_t cur = __ldcg(map + s);
        if (claim_epoch(cur) != epoch) return 0xFFFFFFFFu;
        if (claim_id(cur) == id) return claim_ord(cur);
        s = (s + 1) & mask;
    }
    return 0xFFFFFFFFu;
}

// Slots of digit group g in the reserved pass-1 layout of the segmented
// insert (the host sizes its allocation with it, k_sp_groups the layout):
// the group's expected records (sp.lam[i]: per bucket of table i, rounded
// up) plus 1/64 of them plus two tiles.
__host__ __device__ inline uint64_t sp_group_cap(const SortParams& sp, uint32_t g) {
    const uint32_t b0 = g << sp.hi_shift, b1 = (g + 1) << sp.hi_shift;
    uint64_t lam = 0;
    for (uint32_t i = 0; i < sp.n_tables; ++i) {
        const uint32_t lo = b0 > sp.bbase[i] ? b0 : sp.bbase[i];
        const uint32_t hi = b1 < sp.bbase[i + 1] ? b1 : sp.bbase[i + 1];
        if (hi > lo) lam += (uint64_t)(hi - lo) * sp.lam[i];
    }
    return lam + lam / 64 + 2 * SP_TILE;
}

}  // namespace gdbg
