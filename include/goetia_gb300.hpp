// goetia_gb300.hpp -- header-only C++ front end over the C ABI in goetia_gb300.h.
//
// Restores the reference's C++ signatures for the hot path so goetia's cppyy
// layer (or any C++ caller) can swap it in:
//
//   cppyy.include("goetia_gb300.hpp")
//   cppyy.load_library("libgoetia_gb300.so")
//   g = cppyy.gbl.goetia_gb300.GpuDBG[cppyy.gbl.goetia_gb300.BitStorage,
//                                      cppyy.gbl.goetia_gb300.CanLemireShifter].build(1 << 22, 4, 31)
//
// Mirrors (goetia source tree):
//   dBG<StorageType, ShifterType>      include/goetia/dbg.hh:39-438
//   Storage::build(max_table, N)       include/goetia/storage/bitstorage.hh:69-71
//   UnitigWalker in/out degree         include/goetia/traversal/unitig_walker.hh:322-330
// Errors come back as the reference's exception kinds (same names, in the
// goetia_gb300 namespace): SequenceLengthException, InvalidSequenceException,
// GoetiaException.
#ifndef GOETIA_GB300_HPP
#define GOETIA_GB300_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "goetia_gb300.h"

namespace goetia_gb300 {

typedef int16_t count_t;   // storage.hh:80

struct GoetiaException : std::runtime_error {
    explicit GoetiaException(const std::string& m) : std::runtime_error(m) {}
};
struct SequenceLengthException : GoetiaException {
    explicit SequenceLengthException(const std::string& m) : GoetiaException(m) {}
};
struct InvalidSequenceException : GoetiaException {
    explicit InvalidSequenceException(const std::string& m) : GoetiaException(m) {}
};
struct GoetiaFileException : GoetiaException {   // goetia.hh:155-160
    explicit GoetiaFileException(const std::string& m) : GoetiaException(m) {}
};

inline void check(int rc) {
    if (rc == GDBG_OK) return;
    std::string msg = gdbg_last_error();
    if (rc == GDBG_ERR_SEQUENCE_LENGTH) throw SequenceLengthException(msg);
    if (rc == GDBG_ERR_INVALID_SEQUENCE) throw InvalidSequenceException(msg);
    if (rc == GDBG_ERR_OOM) throw std::bad_alloc();
    if (rc == GDBG_ERR_IO) throw GoetiaFileException(msg);
    throw GoetiaException(msg);
}

// storage / shifter tags
struct BitStorage {
    static constexpr int kind = GDBG_BIT;
    static constexpr bool is_counting = false;
};
struct ByteStorage {
    static constexpr int kind = GDBG_BYTE;
    static constexpr bool is_counting = true;
};
struct NibbleStorage {
    static constexpr int kind = GDBG_NIBBLE;
    static constexpr bool is_counting = true;
};

// Hash<uint64_t> / Canonical<uint64_t> (canonical.hh:30-147)
struct Hash {
    uint64_t hash;
    uint64_t value() const { return hash; }
};
struct Canonical {
    uint64_t fw_hash, rc_hash;
    uint64_t value() const { return fw_hash < rc_hash ? fw_hash : rc_hash; }
    bool sign() const { return fw_hash < rc_hash; }
};
struct FwdLemireShifter {
    static constexpr int kind = GDBG_FWD_LEMIRE;
    typedef Hash hash_type;
    static Hash make(uint64_t v, uint64_t, uint64_t) { return Hash{v}; }
};
struct CanLemireShifter {
    static constexpr int kind = GDBG_CAN_LEMIRE;
    typedef Canonical hash_type;
    static Canonical make(uint64_t, uint64_t fw, uint64_t rc) { return Canonical{fw, rc}; }
};

template <class StorageType, class ShifterType>
class GpuDBG {
    gdbg_graph* g_;
    uint16_t K_;
    explicit GpuDBG(gdbg_graph* g, uint16_t K) : g_(g), K_(K) {}

public:
    typedef typename ShifterType::hash_type hash_type;
    typedef StorageType storage_type;
    typedef ShifterType shifter_type;

    GpuDBG(const GpuDBG&) = delete;
    GpuDBG& operator=(const GpuDBG&) = delete;
    ~GpuDBG() { gdbg_destroy(g_); }

    // Storage::build(max_table, N) + dBG::build(storage, K)
    static std::shared_ptr<GpuDBG> build(uint64_t max_table, uint16_t N, uint16_t K) {
        gdbg_graph* g = nullptr;
        check(gdbg_create(StorageType::kind, ShifterType::kind, K, max_table, N, &g));
        return std::shared_ptr<GpuDBG>(new GpuDBG(g, K));
    }
    static std::shared_ptr<GpuDBG> build(const std::vector<uint64_t>& sizes, uint16_t K) {
        gdbg_graph* g = nullptr;
        check(gdbg_create_sized(StorageType::kind, ShifterType::kind, K, sizes.data(),
                                (uint16_t)sizes.size(), &g));
        return std::shared_ptr<GpuDBG>(new GpuDBG(g, K));
    }
    // dBG::clone (dbg.hh:128-131)
    std::shared_ptr<GpuDBG> clone() const {
        gdbg_graph* g = nullptr;
        check(gdbg_clone(g_, &g));
        return std::shared_ptr<GpuDBG>(new GpuDBG(g, K_));
    }

    uint16_t K() const { return K_; }
    gdbg_graph* handle() const { return g_; }

    hash_type hash(const std::string& kmer) const {
        uint64_t v = 0, fw = 0, rc = 0;
        check(gdbg_hash(g_, kmer.data(), kmer.size(), &v, &fw, &rc));
        return ShifterType::make(v, fw, rc);
    }

    // dBG::insert / query (dbg.hh:140-177)
    bool insert(const hash_type& h) { return insert_value(h.value()); }
    bool insert(const std::string& kmer) { return insert_value(hash(kmer).value()); }
    count_t query(const hash_type& h) { return query_value(h.value()); }
    count_t query(const std::string& kmer) { return query_value(hash(kmer).value()); }
    count_t insert_and_query(const hash_type& h) {
        bool is_new = insert(h);
        if (!StorageType::is_counting) return 1;
        return is_new ? 1 : query(h);
    }

    // dBG::insert_sequence overloads (dbg.hh:249-318)
    uint64_t insert_sequence(const std::string& seq) {
        uint64_t nk = 0;
        check(gdbg_insert_sequence(g_, seq.data(), seq.size(), &nk, nullptr));
        return nk;
    }
    uint64_t insert_sequence(const std::string& seq, uint64_t& n_new) {
        uint64_t nk = 0;
        check(gdbg_insert_sequence(g_, seq.data(), seq.size(), &nk, &n_new));
        return nk;
    }
    uint64_t insert_sequence(const std::string& seq, std::vector<hash_type>& hashes) {
        auto hs = get_hashes(seq);
        std::vector<uint64_t> vals(hs.size());
        for (size_t i = 0; i < hs.size(); ++i) vals[i] = hs[i].value();
        check(gdbg_insert_hashes(g_, vals.data(), vals.size(), nullptr));
        hashes.insert(hashes.end(), hs.begin(), hs.end());
        return seq.size() - K_ + 1;
    }

    uint64_t insert_sequence(const std::string& seq, std::vector<hash_type>& hashes,
                             std::vector<count_t>& counts) {
        auto hs = get_hashes(seq);
        auto c = insert_and_query_sequence(seq);
        hashes.insert(hashes.end(), hs.begin(), hs.end());
        counts.insert(counts.end(), c.begin(), c.end());
        return seq.size() - K_ + 1;
    }
    // dBG::insert_and_query_sequence (dbg.hh:327-340)
    std::vector<count_t> insert_and_query_sequence(const std::string& seq) {
        if (seq.size() < K_) throw SequenceLengthException("Sequence must have length >= K");
        std::vector<count_t> counts(seq.size() - K_ + 1);
        check(gdbg_insert_and_query_sequence(g_, seq.data(), seq.size(), counts.data(), nullptr));
        return counts;
    }

    // dBG::query_sequence (dbg.hh:349-376)
    std::vector<count_t> query_sequence(const std::string& seq) {
        if (seq.size() < K_) throw SequenceLengthException("Sequence must have length >= K");
        std::vector<count_t> counts(seq.size() - K_ + 1);
        check(gdbg_query_sequence(g_, seq.data(), seq.size(), counts.data(), nullptr));
        return counts;
    }
    void query_sequence(const std::string& seq, std::vector<count_t>& counts,
                        std::vector<hash_type>& hashes) {
        auto c = query_sequence(seq);
        auto h = get_hashes(seq);
        counts.insert(counts.end(), c.begin(), c.end());
        hashes.insert(hashes.end(), h.begin(), h.end());
    }

    // the compactor's per-k-mer query (compactor.hh:346-466): flags bit 0 new,
    // bit 1 seen; masks over the storage plus the sequence's new k-mers
    void compactor_query(const std::string& seq, std::vector<uint8_t>& flags,
                         std::vector<uint8_t>& masks) {
        if (seq.size() < K_) throw SequenceLengthException("Sequence must have length >= K");
        flags.assign(seq.size() - K_ + 1, 0);
        masks.assign(seq.size() - K_ + 1, 0);
        check(gdbg_compactor_sequence(g_, seq.data(), seq.size(), flags.data(), masks.data()));
    }

    // get_hash_iter as a vector (dbg.hh:421-425)
    std::vector<hash_type> get_hashes(const std::string& seq) const {
        if (seq.size() < K_) throw SequenceLengthException("Sequence must have length >= K");
        size_t n = seq.size() - K_ + 1;
        std::vector<uint64_t> v(n), fw(n), rc(n);
        check(gdbg_hashes(g_, seq.data(), seq.size(), v.data(), fw.data(), rc.data()));
        std::vector<hash_type> out;
        out.reserve(n);
        for (size_t i = 0; i < n; ++i) out.push_back(ShifterType::make(v[i], fw[i], rc[i]));
        return out;
    }

    // neighbour masks and the walker's degree queries (unitig_walker.hh:322-330)
    std::vector<uint8_t> neighbor_masks(const std::string& seq) {
        if (seq.size() < K_) throw SequenceLengthException("Sequence must have length >= K");
        std::vector<uint8_t> m(seq.size() - K_ + 1);
        check(gdbg_neighbor_masks(g_, seq.data(), seq.size(), m.data()));
        return m;
    }
    size_t in_degree(const std::string& kmer) { return popcount(mask_of(kmer) & 15u); }
    size_t out_degree(const std::string& kmer) { return popcount(mask_of(kmer) >> 4); }
    bool is_decision_kmer(const std::string& kmer) {
        uint8_t m = mask_of(kmer);
        return popcount(m & 15u) > 1 || popcount(m >> 4) > 1;
    }
    // find_decision_kmers positions (unitig_walker.hh:1025-1045)
    std::vector<uint32_t> find_decision_kmers(const std::string& seq) {
        auto m = neighbor_masks(seq);
        std::vector<uint32_t> pos;
        for (size_t i = 0; i < m.size(); ++i)
            if (popcount(m[i] & 15u) > 1 || popcount(m[i] >> 4) > 1) pos.push_back((uint32_t)i);
        return pos;
    }

    uint64_t n_unique() const {
        uint64_t u = 0, o = 0;
        check(gdbg_stats(g_, &u, &o));
        return u;
    }
    uint64_t n_occupied() const {
        uint64_t u = 0, o = 0;
        check(gdbg_stats(g_, &u, &o));
        return o;
    }
    void reset() { check(gdbg_reset(g_)); }
    // BitStorage::update_from (bitstorage.cc:103-137): OR-merge other's tables
    void update_from(const GpuDBG& other) { check(gdbg_update_from(g_, other.g_)); }
    // dBG::save / dBG::load (dbg.hh:396-403): OXLI v4 table files
    void save(const std::string& filename) { check(gdbg_save(g_, filename.c_str())); }
    void load(const std::string& filename) {
        uint16_t ksize = 0;
        check(gdbg_load(g_, filename.c_str(), &ksize));
    }
    std::vector<uint64_t> get_tablesizes() const {
        uint16_t n = 0;
        check(gdbg_info(g_, nullptr, nullptr, nullptr, &n));
        std::vector<uint64_t> s(n);
        check(gdbg_get_tablesizes(g_, s.data()));
        return s;
    }
    // dBG::get_raw, copied out: one byte vector per table in the reference layout
    std::vector<std::vector<uint8_t>> get_raw() const {
        auto sizes = get_tablesizes();
        std::vector<uint64_t> nb(sizes.size());
        check(gdbg_table_bytes(g_, nb.data()));
        uint64_t total = 0;
        for (auto b : nb) total += b;
        std::vector<uint8_t> flat(total);
        check(gdbg_get_tables(g_, flat.data(), total));
        std::vector<std::vector<uint8_t>> out;
        uint64_t pos = 0;
        for (auto b : nb) {
            out.emplace_back(flat.begin() + pos, flat.begin() + pos + b);
            pos += b;
        }
        return out;
    }

private:
    static size_t popcount(unsigned v) {
        size_t c = 0;
        for (; v; v &= v - 1) ++c;
        return c;
    }
    uint8_t mask_of(const std::string& kmer) {
        if (kmer.size() < K_) throw InvalidSequenceException("Sequence must at least length K");
        uint8_t m = 0;
        check(gdbg_neighbor_masks(g_, kmer.data(), K_, &m));
        return m;
    }
    bool insert_value(uint64_t v) {
        uint8_t is_new = 0;
        check(gdbg_insert_hashes(g_, &v, 1, &is_new));
        return is_new != 0;
    }
    count_t query_value(uint64_t v) {
        count_t c = 0;
        check(gdbg_query_hashes(g_, &v, 1, &c));
        return c;
    }
};

}  // namespace goetia_gb300

#endif  // GOETIA_GB300_HPP
