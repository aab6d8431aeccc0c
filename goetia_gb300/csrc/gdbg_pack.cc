// Host-side read packing: text reads -> 2-bit packed stream + base offsets.
//
// The filtering rules are those of goetia's FASTX reader for DNA_SIMPLE
// (FastxParser::next, include/goetia/parsing/readers.hh:150-219, with
// Alphabet::validate, include/goetia/sequences/alphabets.hh:41-56,107-130):
// lowercase acgt are upper-cased, a read holding any other symbol is dropped
// and counted as skipped, and reads shorter than min_length are dropped.
#include <cstdint>
#include <cstring>
#include <string>

#include "goetia_gb300.h"

namespace {
// 0..3 for ACGT/acgt, 4 for anything else
struct CodeTable {
    uint8_t v[256];
    CodeTable() {
        std::memset(v, 4, sizeof v);
        v['A'] = v['a'] = 0;
        v['C'] = v['c'] = 1;
        v['G'] = v['g'] = 2;
        v['T'] = v['t'] = 3;
    }
};
const CodeTable kCodes;
}  // namespace

extern "C" int gdbg_pack_reads(const char* seqs, const uint64_t* so, uint64_t n, uint32_t min_length,
                               uint32_t* packed, uint64_t packed_words, uint64_t* offsets,
                               uint64_t* n_kept, uint64_t* n_skipped) {
    if ((!seqs && n) || !so || !offsets || !n_kept || !n_skipped || (!packed && packed_words))
        return GDBG_ERR_INVALID_ARG;
    uint64_t kept = 0, skipped = 0, pos = 0;
    offsets[0] = 0;
    for (uint64_t r = 0; r < n; ++r) {
        if (so[r + 1] < so[r]) return GDBG_ERR_INVALID_ARG;
        const unsigned char* s = (const unsigned char*)seqs + so[r];
        const uint64_t L = so[r + 1] - so[r];
        bool ok = true;
        for (uint64_t i = 0; i < L && ok; ++i) ok = kCodes.v[s[i]] < 4;
        if (!ok || L < min_length) {
            ++skipped;
            continue;
        }
        if ((pos + L + 15) / 16 > packed_words) return GDBG_ERR_INVALID_ARG;
        for (uint64_t i = 0; i < L; ++i) {
            const uint64_t j = pos + i;
            if ((j & 15u) == 0) packed[j >> 4] = 0;
            packed[j >> 4] |= (uint32_t)kCodes.v[s[i]] << ((j & 15u) << 1);
        }
        pos += L;
        offsets[++kept] = pos;
    }
    *n_kept = kept;
    *n_skipped = skipped;
    return GDBG_OK;
}

extern "C" int gdbg_pack_codes(const uint8_t* codes, uint64_t n, uint32_t* packed) {
    if ((!codes || !packed) && n) return GDBG_ERR_INVALID_ARG;
    const uint64_t full = n / 16;
    for (uint64_t w = 0; w < full; ++w) {
        const uint8_t* c = codes + w * 16;
        uint32_t v = 0;
        for (int i = 0; i < 16; ++i) v |= (uint32_t)(c[i] & 3u) << (2 * i);
        packed[w] = v;
    }
    if (n % 16) {
        uint32_t v = 0;
        for (uint64_t i = full * 16; i < n; ++i) v |= (uint32_t)(codes[i] & 3u) << (2 * (i & 15u));
        packed[full] = v;
    }
    return GDBG_OK;
}
