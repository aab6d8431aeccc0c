// Golden-vector driver for the reference goetia C++ hot path.
//
// Test infrastructure only: this program links the reference's own objects
// (built by oracle/Makefile from the read-only reference sources into
// oracle/_ref/) and writes the reference's answers for a set of reads, so the
// C restatement in oracle/goetia_oracle.c and the CUDA library can be pinned
// against the real thing.  Nothing in the product links or runs it.
//
// Usage:
//   ref_driver <bit|byte|nibble> <can|fwd> <K> <n_tables> <max_table> <reads.txt> <outdir>
//   ref_driver time <bit|byte|nibble> <can|fwd> <K> <n_tables> <max_table> <reads.txt>
//
// The second form only times dBG::insert_sequence(seq, n_new) over the reads
// in file order on one thread (steady clock around the loop) and prints
// "<k-mers> <new k-mers> <seconds>", for comparing the C restatement's speed
// with the reference's own code on the same host.
//
// reads.txt holds one read per line.  For every read, in file order, the
// driver calls dBG::insert_sequence(seq, n_new) (dbg.hh:296-305), catching the
// SequenceLengthException thrown for reads shorter than K the way
// InserterProcessor does (processors.hh:304-331).  After all inserts it
// records, per k-mer of every read:
//   - the hash from get_hash_iter (dbg.hh:421-425), fw/rc for canonical;
//   - query_sequence counts (dbg.hh:349-362);
//   - an 8-bit neighbour mask: bit i = left extension "ACGT"[i] present,
//     bit 4+i = right extension present, from set_cursor + left/right_extensions
//     + query (hashextender.hh:352-396, unitig_walker.hh:361-397);
// plus find_decision_kmers positions (unitig_walker.hh:1025-1045), the raw
// table bytes (get_raw), n_unique / n_occupied, and the OXLI file written by
// dBG::save (dbg.hh:396-398 -> Storage::save, bitstorage.cc:151-186,
// bytestorage.cc:480-521, nibblestorage.cc:132-166) as saved.oxli, the
// insert_and_query_sequence counts of all reads on fresh tables, and for
// Bit storages the tables and counters after BitStorage::update_from
// (bitstorage.cc:103-137) of two half-read graphs.
#include "goetia/dbg.hh"
#include "goetia/storage/bitstorage.hh"
#include "goetia/storage/bytestorage.hh"
#include "goetia/storage/nibblestorage.hh"
#include "goetia/hashing/shifter_types.hh"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <type_traits>
#include <vector>

using namespace goetia;

template <class T>
static void dump(const std::string& path, const std::vector<T>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

template <class T> static uint64_t fw_of(const T& h);
template <> uint64_t fw_of(const Canonical<uint64_t>& h) { return h.fw_hash; }
template <> uint64_t fw_of(const Hash<uint64_t>& h) { return h.value(); }
template <class T> static uint64_t rc_of(const T& h);
template <> uint64_t rc_of(const Canonical<uint64_t>& h) { return h.rc_hash; }
template <> uint64_t rc_of(const Hash<uint64_t>& h) { return 0; }

template <class Storage, class Shifter>
static int run(uint16_t K, uint16_t n_tables, uint64_t max_table,
               const std::vector<std::string>& reads, const std::string& out) {
    auto storage = Storage::build(max_table, n_tables);
    auto graph = dBG<Storage, Shifter>::build(storage, K);
    using hash_type = typename dBG<Storage, Shifter>::hash_type;

    std::vector<uint64_t> n_new(reads.size(), 0), n_kmers(reads.size(), 0);
    for (size_t r = 0; r < reads.size(); ++r) {
        try {
            uint64_t nn = 0;
            n_kmers[r] = graph->insert_sequence(reads[r], nn);
            n_new[r] = nn;
        } catch (SequenceLengthException&) {
            n_kmers[r] = 0;
            n_new[r] = 0;
        }
    }

    std::vector<uint64_t> fw, rc, val, dpos_read, dpos_pos;
    std::vector<int16_t> counts;
    std::vector<uint8_t> masks;
    for (size_t r = 0; r < reads.size(); ++r) {
        const std::string& s = reads[r];
        if (s.size() < K) continue;
        auto it = graph->get_hash_iter(s);
        while (!it->done()) {
            hash_type h = it->next();
            fw.push_back(fw_of(h));
            rc.push_back(rc_of(h));
            val.push_back(h.value());
        }
        auto c = graph->query_sequence(s);
        counts.insert(counts.end(), c.begin(), c.end());
        for (size_t p = 0; p + K <= s.size(); ++p) {
            graph->set_cursor(s.substr(p, K));
            auto left = graph->left_extensions();
            auto right = graph->right_extensions();
            uint8_t m = 0;
            for (size_t i = 0; i < left.size(); ++i)
                if (graph->query(left[i])) m |= (uint8_t)(1u << i);
            for (size_t i = 0; i < right.size(); ++i)
                if (graph->query(right[i])) m |= (uint8_t)(1u << (4 + i));
            masks.push_back(m);
        }
        std::vector<uint32_t> positions;
        std::vector<hash_type> dhashes;
        std::vector<typename dBG<Storage, Shifter>::neighbor_pair_type> neighbors;
        graph->find_decision_kmers(s, positions, dhashes, neighbors);
        for (auto p : positions) { dpos_read.push_back(r); dpos_pos.push_back(p); }
    }

    auto sizes = storage->get_tablesizes();
    dump(out + "/sizes.u64", sizes);
    dump(out + "/n_new.u64", n_new);
    dump(out + "/n_kmers.u64", n_kmers);
    dump(out + "/fw.u64", fw);
    dump(out + "/rc.u64", rc);
    dump(out + "/val.u64", val);
    dump(out + "/counts.i16", counts);
    dump(out + "/masks.u8", masks);
    dump(out + "/dpos_read.u64", dpos_read);
    dump(out + "/dpos_pos.u64", dpos_pos);
    uint8_t** raw = graph->get_raw();
    for (size_t i = 0; i < sizes.size(); ++i) {
        uint64_t nbytes = std::is_same<Storage, BitStorage>::value ? sizes[i] / 8 + 1
                        : std::is_same<Storage, NibbleStorage>::value ? sizes[i] / 2 + 1
                        : sizes[i];
        std::vector<uint8_t> t(raw[i], raw[i] + nbytes);
        dump(out + "/table" + std::to_string(i) + ".u8", t);
    }
    std::vector<uint64_t> stats = {graph->n_unique(), graph->n_occupied()};
    dump(out + "/stats.u64", stats);
    graph->save(out + "/saved.oxli");

    // dBG::insert_and_query_sequence (dbg.hh:327-340) per read on fresh tables
    {
        auto s2 = Storage::build(max_table, n_tables);
        auto g2 = dBG<Storage, Shifter>::build(s2, K);
        std::vector<int16_t> iq;
        for (const auto& s : reads) {
            if (s.size() < K) continue;
            auto c = g2->insert_and_query_sequence(s);
            iq.insert(iq.end(), c.begin(), c.end());
        }
        dump(out + "/iq_counts.i16", iq);
    }

    // Compactor query (compactor.hh:346-466 with filter_nodes and extras,
    // unitig_walker.hh:457-469): graph H holds the first half of the reads;
    // every k-mer of the second half gets new = query() == 0, seen = already
    // in the read's new-k-mer set, and its neighbour mask over the storage
    // plus the read's new k-mers.
    {
        auto sh = Storage::build(max_table, n_tables);
        auto gh = dBG<Storage, Shifter>::build(sh, K);
        const size_t half = reads.size() / 2;
        for (size_t r = 0; r < half; ++r)
            if (reads[r].size() >= K) gh->insert_sequence(reads[r]);
        std::vector<uint8_t> cflags, cmasks;
        auto sym_index = [](char c) { return c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3; };
        for (size_t r = half; r < reads.size(); ++r) {
            const std::string& s = reads[r];
            if (s.size() < K) continue;
            std::set<hash_type> new_kmers;
            auto it = gh->get_hash_iter(s);
            while (!it->done()) {
                hash_type h = it->next();
                const bool cur_new = gh->query(h) == 0;
                const bool cur_seen = new_kmers.count(h) > 0;
                if (cur_new && !cur_seen) new_kmers.insert(h);
                cflags.push_back((uint8_t)((cur_new ? 1 : 0) | (cur_seen ? 2 : 0)));
            }
            for (size_t p = 0; p + K <= s.size(); ++p) {
                gh->set_cursor(s.substr(p, K));
                auto left = gh->filter_nodes(gh->left_extensions(), new_kmers);
                auto right = gh->filter_nodes(gh->right_extensions(), new_kmers);
                uint8_t m = 0;
                for (auto& e : left) m |= (uint8_t)(1u << sym_index(e.symbol));
                for (auto& e : right) m |= (uint8_t)(1u << (4 + sym_index(e.symbol)));
                cmasks.push_back(m);
            }
        }
        dump(out + "/compactor_flags.u8", cflags);
        dump(out + "/compactor_masks.u8", cmasks);
    }

    // BitStorage::update_from (bitstorage.cc:103-137): graph A holds the first
    // half of the reads, graph B the second half; A |= B.
    if constexpr (std::is_same<Storage, BitStorage>::value) {
        auto sa = Storage::build(max_table, n_tables), sb = Storage::build(max_table, n_tables);
        auto ga = dBG<Storage, Shifter>::build(sa, K), gb = dBG<Storage, Shifter>::build(sb, K);
        for (size_t r = 0; r < reads.size(); ++r) {
            if (reads[r].size() < K) continue;
            (r < reads.size() / 2 ? ga : gb)->insert_sequence(reads[r]);
        }
        std::vector<uint64_t> pre = {ga->n_unique(), ga->n_occupied(), gb->n_unique(), gb->n_occupied()};
        sa->update_from(*sb);
        pre.push_back(ga->n_unique());
        pre.push_back(ga->n_occupied());
        dump(out + "/merge_stats.u64", pre);
        uint8_t** mraw = ga->get_raw();
        std::vector<uint8_t> merged;
        for (size_t i = 0; i < sizes.size(); ++i)
            merged.insert(merged.end(), mraw[i], mraw[i] + sizes[i] / 8 + 1);
        dump(out + "/merged.u8", merged);
    }
    return 0;
}

template <class Storage, class Shifter>
static int time_insert(uint16_t K, uint16_t n_tables, uint64_t max_table,
                       const std::vector<std::string>& reads) {
    auto storage = Storage::build(max_table, n_tables);
    auto graph = dBG<Storage, Shifter>::build(storage, K);
    uint64_t total = 0, new_total = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (const auto& s : reads) {
        try {
            uint64_t nn = 0;
            total += graph->insert_sequence(s, nn);
            new_total += nn;
        } catch (SequenceLengthException&) {
        }
    }
    const double dt =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("%llu %llu %.6f\n", (unsigned long long)total, (unsigned long long)new_total, dt);
    return 0;
}

static std::vector<std::string> read_lines(const char* path) {
    std::vector<std::string> reads;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) reads.push_back(line);
    return reads;
}

int main(int argc, char** argv) {
    if (argc == 8 && std::string(argv[1]) == "time") {
        const std::string kind = argv[2];
        const bool can = std::string(argv[3]) == "can";
        const uint16_t K = (uint16_t)std::atoi(argv[4]);
        const uint16_t N = (uint16_t)std::atoi(argv[5]);
        const uint64_t max_table = std::strtoull(argv[6], nullptr, 10);
        const auto reads = read_lines(argv[7]);
        if (kind == "bit")
            return can ? time_insert<BitStorage, CanLemireShifter>(K, N, max_table, reads)
                       : time_insert<BitStorage, FwdLemireShifter>(K, N, max_table, reads);
        if (kind == "byte")
            return can ? time_insert<ByteStorage, CanLemireShifter>(K, N, max_table, reads)
                       : time_insert<ByteStorage, FwdLemireShifter>(K, N, max_table, reads);
        if (kind == "nibble")
            return can ? time_insert<NibbleStorage, CanLemireShifter>(K, N, max_table, reads)
                       : time_insert<NibbleStorage, FwdLemireShifter>(K, N, max_table, reads);
        std::fprintf(stderr, "unknown storage %s\n", kind.c_str());
        return 1;
    }
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s <bit|byte|nibble> <can|fwd> <K> <n_tables> <max_table> <reads.txt> <outdir>\n", argv[0]);
        return 1;
    }
    std::string kind = argv[1], shifter = argv[2];
    uint16_t K = (uint16_t)std::atoi(argv[3]);
    uint16_t N = (uint16_t)std::atoi(argv[4]);
    uint64_t max_table = std::strtoull(argv[5], nullptr, 10);
    std::vector<std::string> reads;
    std::ifstream in(argv[6]);
    std::string line;
    while (std::getline(in, line)) reads.push_back(line);
    std::string out = argv[7];
    bool can = shifter == "can";
    if (kind == "bit")
        return can ? run<BitStorage, CanLemireShifter>(K, N, max_table, reads, out)
                   : run<BitStorage, FwdLemireShifter>(K, N, max_table, reads, out);
    if (kind == "byte")
        return can ? run<ByteStorage, CanLemireShifter>(K, N, max_table, reads, out)
                   : run<ByteStorage, FwdLemireShifter>(K, N, max_table, reads, out);
    if (kind == "nibble")
        return can ? run<NibbleStorage, CanLemireShifter>(K, N, max_table, reads, out)
                   : run<NibbleStorage, FwdLemireShifter>(K, N, max_table, reads, out);
    std::fprintf(stderr, "unknown storage %s\n", kind.c_str());
    return 1;
}
