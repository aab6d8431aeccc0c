// Seeded synthetic read generator for the benchmark workloads (host, C++,
// multi-threaded): the data-loader stand-in that feeds the batched and
// serving legs with billions of bases in seconds.  It is not part of the
// insert path and has no counterpart in the reference (whose inputs are
// FASTA/FASTQ files); no public dataset is involved.
//
// Every random choice is a pure function of (seed, read, position) -- a
// splitmix64-style mix, the same in goetia_gb300/synth.py's numpy twin -- so
// any read can be regenerated alone, and the output does not depend on the
// number of threads.  Codes: A=0 C=1 G=2 T=3; output is the library's packed
// stream (base j in bits 2*(j%16) of uint32 word j/16) plus base offsets.
//
//   wl_sample_reads: reads of one fixed length from one genome, uniform
//       start, either strand, i.i.d. substitutions;
//   wl_uneven_lengths / wl_uneven_write: reads with caller-chosen source
//       windows (genome, start, length, strand), every source base deleted,
//       substituted, or followed by an inserted random base, at given rates.
#include <atomic>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

namespace {

inline uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// per-read stream key, then one draw per position
inline uint64_t read_key(uint64_t seed, uint64_t read) { return seed ^ mix(read + 0x9E3779B97F4A7C15ull); }
inline uint64_t draw(uint64_t key, uint64_t pos) { return mix(key ^ (pos * 0xD6E8FEB86659FD93ull)); }

constexpr uint64_t POS_START = 1ull << 40;   // draw positions of per-read choices
constexpr uint64_t POS_STRAND = (1ull << 40) + 1;

inline uint32_t threshold(double rate) {   // rate as a 24-bit fraction
    double t = rate * (double)(1u << 24);
    if (t < 0) t = 0;
    if (t > (double)(1u << 24)) t = (double)(1u << 24);
    return (uint32_t)(t + 0.5);
}

// Writes 2-bit codes into a zeroed packed stream from one thread; the words
// at either end of its range may be shared with a neighbour's range, so they
// are OR-ed atomically.
struct PackedWriter {
    uint32_t* out;
    uint64_t first_w, last_w, w, pos;
    uint32_t v;
    PackedWriter(uint32_t* o, uint64_t begin, uint64_t end)
        : out(o), first_w(begin >> 4), last_w(end ? (end - 1) >> 4 : 0), w(begin >> 4), pos(begin), v(0) {}
    void flush() {
        if (!v) return;
        if (w == first_w || w == last_w) __atomic_fetch_or(out + w, v, __ATOMIC_RELAXED);
        else out[w] = v;
        v = 0;
    }
    void put(uint32_t c) {
        const uint64_t ww = pos >> 4;
        if (ww != w) {
            flush();
            w = ww;
        }
        v |= (c & 3u) << ((pos & 15u) << 1);
        ++pos;
    }
    ~PackedWriter() { flush(); }
};

// Contiguous read ranges of about equal weight (bases) per thread.
std::vector<uint64_t> split(const uint64_t* weight_prefix, uint64_t n, int threads) {
    std::vector<uint64_t> cut(threads + 1, n);
    cut[0] = 0;
    const uint64_t total = weight_prefix[n];
    uint64_t r = 0;
    for (int t = 1; t < threads; ++t) {
        const uint64_t want = total / threads * t;
        while (r < n && weight_prefix[r] < want) ++r;
        cut[t] = r;
    }
    return cut;
}

template <class F>
void parallel(int threads, F&& f) {
    if (threads < 1) threads = 1;
    std::vector<std::thread> th;
    for (int t = 1; t < threads; ++t) th.emplace_back(f, t);
    f(0);
    for (auto& x : th) x.join();
}

inline uint32_t src_base(const uint8_t* g, uint64_t start, uint64_t len, bool flip, uint64_t j) {
    return flip ? 3u - (g[start + len - 1 - j] & 3u) : (g[start + j] & 3u);
}

}  // namespace

extern "C" {

// n_reads reads of `length` bases from genome g (glen bases): read r starts at
// draw(r, POS_START) % (glen - length + 1), is reverse-complemented when the
// top bit of draw(r, POS_STRAND) is set, and each base j is substituted (to
// (b + 1 + (x >> 8) % 3) & 3) when (x >> 40) < sub threshold, x = draw(r, j).
// packed must hold n_reads*length/16 + 1 zeroed words; offsets n_reads + 1.
int wl_sample_reads(const uint8_t* g, uint64_t glen, uint64_t n_reads, uint32_t length,
                    uint64_t seed, double sub_rate, uint64_t first_read, uint32_t* packed,
                    uint64_t* offsets, int threads) {
    if (!g || length == 0 || glen < length || (n_reads && (!packed || !offsets))) return 1;
    const uint32_t ts = threshold(sub_rate);
    const uint64_t span = glen - length + 1;
    for (uint64_t r = 0; r <= n_reads; ++r) offsets[r] = r * (uint64_t)length;
    if (threads < 1) threads = 1;
    parallel(threads, [&](int t) {
        const uint64_t r0 = n_reads * t / threads, r1 = n_reads * (t + 1) / threads;
        if (r0 >= r1) return;
        PackedWriter wr(packed, r0 * length, r1 * length);
        for (uint64_t r = r0; r < r1; ++r) {
            const uint64_t key = read_key(seed, first_read + r);
            const uint64_t start = draw(key, POS_START) % span;
            const bool flip = (draw(key, POS_STRAND) >> 63) != 0;
            for (uint32_t j = 0; j < length; ++j) {
                uint32_t b = src_base(g, start, length, flip, j);
                const uint64_t x = draw(key, j);
                if ((uint32_t)(x >> 40) < ts) b = (b + 1u + (uint32_t)((x >> 8) % 3u)) & 3u;
                wr.put(b);
            }
        }
    });
    return 0;
}

// Uneven reads: read r copies src_len[r] bases of genome src_genome[r] from
// src_start[r] (reverse-complemented when flip[r]); each source base j, with
// x = draw(r, j) and u = x >> 40, is deleted when u < del, substituted when
// u < del + sub, followed by the random base (x >> 16) & 3 when
// u < del + sub + ins, kept otherwise.  Pass 1 (wl_uneven_lengths) gives the
// output length of every read; the caller turns them into offsets and calls
// pass 2 (wl_uneven_write) with a zeroed packed buffer of offsets[n]/16 + 1
// words.
static int uneven(bool write, const uint8_t* genomes, const uint64_t* genome_off,
                  uint32_t n_genomes, const uint32_t* src_genome, const uint64_t* src_start,
                  const uint32_t* src_len, const uint8_t* flip, uint64_t n_reads, uint64_t seed,
                  double sub, double ins, double del, uint64_t first_read, uint64_t* out_len,
                  const uint64_t* offsets, uint32_t* packed, int threads) {
    if (!genomes || !genome_off || (n_reads && (!src_genome || !src_start || !src_len || !flip)))
        return 1;
    for (uint64_t r = 0; r < n_reads; ++r) {
        if (src_genome[r] >= n_genomes) return 1;
        const uint64_t gl = genome_off[src_genome[r] + 1] - genome_off[src_genome[r]];
        if (src_start[r] + src_len[r] > gl) return 1;
    }
    const uint32_t td = threshold(del), tsd = threshold(del + sub), tisd = threshold(del + sub + ins);
    std::vector<uint64_t> wp(n_reads + 1, 0);
    for (uint64_t r = 0; r < n_reads; ++r) wp[r + 1] = wp[r] + src_len[r] + 1;
    if (threads < 1) threads = 1;
    const std::vector<uint64_t> cut = split(wp.data(), n_reads, threads);
    parallel(threads, [&](int t) {
        const uint64_t r0 = cut[t], r1 = cut[t + 1];
        if (r0 >= r1) return;
        PackedWriter* wr = nullptr;
        alignas(PackedWriter) unsigned char buf[sizeof(PackedWriter)];
        if (write) wr = new (buf) PackedWriter(packed, offsets[r0], offsets[r1]);
        for (uint64_t r = r0; r < r1; ++r) {
            const uint8_t* g = genomes + genome_off[src_genome[r]];
            const uint64_t key = read_key(seed, first_read + r);
            const uint64_t s0 = src_start[r], L = src_len[r];
            const bool fl = flip[r] != 0;
            uint64_t n = 0;
            for (uint64_t j = 0; j < L; ++j) {
                const uint64_t x = draw(key, j);
                const uint32_t u = (uint32_t)(x >> 40);
                if (u < td) continue;
                uint32_t b = src_base(g, s0, L, fl, j);
                if (u < tsd) b = (b + 1u + (uint32_t)((x >> 8) % 3u)) & 3u;
                if (write) wr->put(b);
                ++n;
                if (u >= tsd && u < tisd) {
                    if (write) wr->put((uint32_t)(x >> 16) & 3u);
                    ++n;
                }
            }
            if (!write) out_len[r] = n;
        }
        if (wr) wr->~PackedWriter();
    });
    return 0;
}

int wl_uneven_lengths(const uint8_t* genomes, const uint64_t* genome_off, uint32_t n_genomes,
                      const uint32_t* src_genome, const uint64_t* src_start, const uint32_t* src_len,
                      const uint8_t* flip, uint64_t n_reads, uint64_t seed, double sub, double ins,
                      double del, uint64_t first_read, uint64_t* out_len, int threads) {
    if (n_reads && !out_len) return 1;
    return uneven(false, genomes, genome_off, n_genomes, src_genome, src_start, src_len, flip,
                  n_reads, seed, sub, ins, del, first_read, out_len, nullptr, nullptr, threads);
}

int wl_uneven_write(const uint8_t* genomes, const uint64_t* genome_off, uint32_t n_genomes,
                    const uint32_t* src_genome, const uint64_t* src_start, const uint32_t* src_len,
                    const uint8_t* flip, uint64_t n_reads, uint64_t seed, double sub, double ins,
                    double del, uint64_t first_read, const uint64_t* offsets, uint32_t* packed,
                    int threads) {
    if (n_reads && (!offsets || !packed)) return 1;
    return uneven(true, genomes, genome_off, n_genomes, src_genome, src_start, src_len, flip,
                  n_reads, seed, sub, ins, del, first_read, nullptr, offsets, packed, threads);
}

}  // extern "C"
