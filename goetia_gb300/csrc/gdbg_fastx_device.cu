// FASTA / FASTQ text in device memory -> records -> the device packer, with
// the results of goetia's FastxParser<DNA_SIMPLE>::next called until the end
// (include/goetia/parsing/readers.hh:150-219) over its vendored kseq reader
// (include/goetia/parsing/kseq.h:88-220).
//
// kseq is a sequential state machine; its records are found in parallel here
// for the two regular layouts, where its result follows from each line alone:
//   FASTQ  every record four lines: '@' header, one sequence line (empty, or
//          not starting with '>', '+' or '@'), a '+' line, one quality line
//          as long as the sequence (kseq reads quality lines until it has
//          the sequence's length, so one line of exactly that length is the
//          whole quality string);
//   FASTA  no line starts with '+'; lines starting with '>' or '@' are
//          headers, every other line belongs to the sequence of the header
//          above it (blank lines add nothing, nor does a lone '\r' line under
//          a sequence line with bytes; a lone '\r' that ends the text is
//          kept; a lone '\r' line anywhere else is refused);
// in both the text starts with the header character and does not end in a
// one-byte header line.  Sequences are the lines' bytes less one trailing
// '\r' (ks_getuntil2 drops it from a line string longer than one byte; a
// FASTQ sequence line of just '\r' keeps it, so that read is dropped as
// invalid, as in kseq).  Any other text (several quality lines, junk before
// the first header, blank lines after a FASTQ record ...) returns
// GDBG_ERR_UNSUPPORTED naming the first line that breaks the layout, and
// the caller parses it on the host.
//
//   k_fx_count     newlines per tile of FX_TILE bytes
//   scan           tile newline bases
//   k_fx_lines     each newline's position, in order
//   k_fx_classify  per line: header flag, sequence bytes (clen), layout check
//   scans          sequence byte offsets (cpos), record index of each header
//   k_fx_spans     FASTQ: each record's sequence as a span of the text
//   k_fx_gather    FASTA: one warp per sequence line, its bytes to the
//                  compacted sequence buffer; each header writes its
//                  record's start
//   pack_device_run  the packer's drop policy and 2-bit packing
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gdbg_launch.h"
#include "goetia_gb300.h"

namespace gdbg {

constexpr int FX_BLOCK = 256;
constexpr uint32_t FX_SEG = 32;                    // bytes per thread
constexpr uint32_t FX_TILE = FX_BLOCK * FX_SEG;    // bytes per block

// The thread's FX_SEG bytes from `base` (bytes past n read as 0); vector
// loads when the text is 16-byte aligned and the segment is whole.
template <bool ALIGNED>
__device__ __forceinline__ void fx_load(const unsigned char* __restrict__ text, uint64_t base,
                                        uint64_t n, uint32_t w[FX_SEG / 4]) {
    if (ALIGNED && base + FX_SEG <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(text + base);
        const uint4 a = __ldg(p), b = __ldg(p + 1);
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
        w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
        return;
    }
#pragma unroll
    for (uint32_t q = 0; q < FX_SEG / 4; ++q) {
        uint32_t v = 0;
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            const uint64_t j = base + q * 4 + k;
            if (j < n) v |= (uint32_t)__ldg(text + j) << (8 * k);
        }
        w[q] = v;
    }
}

// bit k*8 of the result set where byte k of v is '\n'
__device__ __forceinline__ uint32_t fx_nl_bits(uint32_t v) {
    return __vcmpeq4(v, 0x0A0A0A0Au) & 0x01010101u;
}

template <bool ALIGNED>
__global__ void __launch_bounds__(FX_BLOCK)
k_fx_count(const unsigned char* __restrict__ text, uint64_t n, uint32_t* __restrict__ tile_cnt) {
    __shared__ uint32_t ws[FX_BLOCK / 32];
    const uint64_t base = (uint64_t)blockIdx.x * FX_TILE + (uint64_t)threadIdx.x * FX_SEG;
    uint32_t w[FX_SEG / 4];
    fx_load<ALIGNED>(text, base, n, w);
    uint32_t c = 0;
#pragma unroll
    for (uint32_t q = 0; q < FX_SEG / 4; ++q) c += __popc(fx_nl_bits(w[q]));
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int k = 0; k < FX_BLOCK / 32; ++k) t += ws[k];
        tile_cnt[blockIdx.x] = t;
    }
}

template <bool ALIGNED>
__global__ void __launch_bounds__(FX_BLOCK)
k_fx_lines(const unsigned char* __restrict__ text, uint64_t n, const uint32_t* __restrict__ tile_base,
           uint32_t* __restrict__ nlpos, uint32_t n_nl) {
    __shared__ uint32_t ws[FX_BLOCK / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint64_t base = (uint64_t)blockIdx.x * FX_TILE + (uint64_t)tid * FX_SEG;
    uint32_t w[FX_SEG / 4];
    fx_load<ALIGNED>(text, base, n, w);
    uint32_t c = 0;
#pragma unroll
    for (uint32_t q = 0; q < FX_SEG / 4; ++q) c += __popc(fx_nl_bits(w[q]));
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    uint32_t pre = 0;
    for (uint32_t k = 0; k < wid; ++k) pre += ws[k];
    uint32_t idx = tile_base[blockIdx.x] + pre + inc - c;
#pragma unroll
    for (uint32_t q = 0; q < FX_SEG / 4; ++q) {
        uint32_t m = fx_nl_bits(w[q]);
        while (m) {
            const uint32_t k = (uint32_t)(__ffs(m) - 1) >> 3;
            m &= m - 1;
            if (idx < n_nl) nlpos[idx] = (uint32_t)(base + q * 4 + k);
            ++idx;
        }
    }
}

// Line j: [start, end) without its '\n'.
__device__ __forceinline__ void fx_line(const uint32_t* __restrict__ nlpos, uint32_t n_nl, uint64_t n,
                                        uint32_t j, uint64_t& start, uint64_t& end) {
    start = j == 0 ? 0 : (uint64_t)nlpos[j - 1] + 1;
    end = j < n_nl ? nlpos[j] : n;
}

// Sequence bytes of a line: its length less one trailing '\r' when longer
// than one byte.
__device__ __forceinline__ uint32_t fx_eff_len(const unsigned char* __restrict__ text, uint64_t start,
                                               uint64_t end) {
    const uint64_t len = end - start;
    return (uint32_t)(len - ((len >= 2 && text[end - 1] == '\r') ? 1 : 0));
}

// mode: 1 FASTQ (the text starts with '@' and its third line with '+'),
// 0 FASTA.  bad gets the smallest line index that breaks the layout.
__global__ void __launch_bounds__(FX_BLOCK)
k_fx_classify(const unsigned char* __restrict__ text, uint64_t n, const uint32_t* __restrict__ nlpos,
              uint32_t n_nl, uint32_t n_lines, uint32_t* __restrict__ clen, uint32_t* __restrict__ hflag,
              uint32_t* __restrict__ bad, uint32_t* __restrict__ mode_out) {
    const uint32_t j = blockIdx.x * FX_BLOCK + threadIdx.x;
    if (j >= n_lines) return;
    uint32_t mode = 0;
    if (text[0] == '@' && n_lines >= 3) {
        uint64_t s2, e2;
        fx_line(nlpos, n_nl, n, 2, s2, e2);
        mode = (e2 > s2 && text[s2] == '+') ? 1u : 0u;
    }
    if (j == 0) *mode_out = mode;
    uint64_t s, e;
    fx_line(nlpos, n_nl, n, j, s, e);
    const uint64_t len = e - s;
    const int c0 = len ? text[s] : -1;
    bool ok = true;
    uint32_t cl = 0, hf = 0;
    if (mode) {
        const uint32_t role = j & 3u;
        if ((n_lines & 3u) != 0) ok = false;
        if (role == 0) {
            ok = ok && c0 == '@';
            hf = 1;
        } else if (role == 1) {
            ok = ok && c0 != '>' && c0 != '+' && c0 != '@';
            cl = fx_eff_len(text, s, e);
        } else if (role == 2) {
            ok = ok && c0 == '+';
        } else {
            uint64_t ss, se;
            fx_line(nlpos, n_nl, n, j - 2, ss, se);
            ok = ok && fx_eff_len(text, s, e) == fx_eff_len(text, ss, se);
        }
    } else {
        const bool header = c0 == '>' || c0 == '@';
        if (j == 0 && !header) ok = false;
        if (c0 == '+') ok = false;
        // a header byte that ends the text is no record for kseq
        if (header && len == 1 && j >= n_nl) ok = false;
        hf = header ? 1u : 0u;
        cl = header ? 0u : fx_eff_len(text, s, e);
        if (len == 1 && c0 == '\r' && j < n_nl) {
            // kseq drops the '\r' when the sequence above already has bytes:
            // taken when the line above is a sequence line with bytes.  (A
            // lone '\r' that ends the text stays, cl = 1: kseq's read of the
            // rest of that line meets the end of the text and returns before
            // it would drop it, so the read is dropped as invalid.)
            cl = 0;
            if (j == 0) {
                ok = false;
            } else {
                uint64_t ps, pe;
                fx_line(nlpos, n_nl, n, j - 1, ps, pe);
                const int p0 = pe > ps ? text[ps] : -1;
                if (pe == ps || p0 == '>' || p0 == '@' || (pe - ps == 1 && p0 == '\r')) ok = false;
            }
        }
    }
    clen[j] = cl;
    hflag[j] = hf;
    if (!ok) atomicMin(bad, j);
}

// One warp per line: a sequence line's bytes to seqs[cpos[j] ...); a header
// line's record starts at cpos[j] (its own clen is 0).
__global__ void __launch_bounds__(FX_BLOCK)
k_fx_gather(const unsigned char* __restrict__ text, uint64_t n, const uint32_t* __restrict__ nlpos,
            uint32_t n_nl, uint32_t n_lines, const uint32_t* __restrict__ clen,
            const uint32_t* __restrict__ cpos, const uint32_t* __restrict__ hflag,
            const uint32_t* __restrict__ hidx, unsigned char* __restrict__ seqs,
            uint64_t* __restrict__ so) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_warps = (uint64_t)gridDim.x * FX_BLOCK / 32;
    for (uint64_t j = ((uint64_t)blockIdx.x * FX_BLOCK + threadIdx.x) / 32; j < n_lines; j += n_warps) {
        if (hflag[j]) {
            if (lane == 0) so[hidx[j]] = cpos[j];
            continue;
        }
        const uint32_t L = clen[j];
        if (!L) continue;
        uint64_t s, e;
        fx_line(nlpos, n_nl, n, (uint32_t)j, s, e);
        unsigned char* dst = seqs + cpos[j];
        for (uint32_t i = lane; i < L; i += 32) dst[i] = text[s + i];
    }
}

// FASTQ: record r's sequence is one span of the text (line 4r + 1 less a
// trailing '\r'), handed to the packer in place.
__global__ void __launch_bounds__(FX_BLOCK)
k_fx_spans(const unsigned char* __restrict__ text, uint64_t n, const uint32_t* __restrict__ nlpos,
           uint32_t n_nl, uint64_t n_rec, uint64_t* __restrict__ starts, uint64_t* __restrict__ ends) {
    const uint64_t r = (uint64_t)blockIdx.x * FX_BLOCK + threadIdx.x;
    if (r >= n_rec) return;
    uint64_t s, e;
    fx_line(nlpos, n_nl, n, (uint32_t)(4 * r + 1), s, e);
    starts[r] = s;
    ends[r] = s + fx_eff_len(text, s, e);
}

__global__ void k_fx_tail(const uint32_t* clen, const uint32_t* cpos, const uint32_t* hflag,
                          const uint32_t* hidx, uint32_t n_lines, uint64_t* out) {
    out[0] = (uint64_t)cpos[n_lines - 1] + clen[n_lines - 1];   // sequence bytes
    out[1] = (uint64_t)hidx[n_lines - 1] + hflag[n_lines - 1];  // records
}

}  // namespace gdbg

using namespace gdbg;

extern "C" int gdbg_parse_fastx_device(const char* text, uint64_t n_bytes, uint32_t min_length,
                                       uint32_t* packed, uint64_t packed_words, uint64_t* offsets,
                                       uint64_t offsets_cap, uint64_t* stats, void* stream) {
    if (!stats || (!text && n_bytes) || (!packed && packed_words) || (!offsets && offsets_cap))
        return report_error(GDBG_ERR_INVALID_ARG, "NULL argument");
    if (n_bytes >= 0xFFFFFFFFull)
        return report_error(GDBG_ERR_INVALID_ARG, "text of 2^32 - 1 bytes or more: split it at a record boundary");
    for (int i = 0; i < 4; ++i) stats[i] = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned char* t = (const unsigned char*)text;
    if (n_bytes == 0) {
        if (!offsets_cap) return report_error(GDBG_ERR_INVALID_ARG, "offsets needs 1 entry");
        const uint64_t zero = 0;
        cudaError_t e = cudaMemcpyAsync(offsets, &zero, sizeof zero, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? GDBG_OK : report_error(GDBG_ERR_CUDA, cudaGetErrorString(e));
    }
    const bool aligned = ((uintptr_t)text & 15u) == 0;
    const uint64_t n_tiles = (n_bytes + FX_TILE - 1) / FX_TILE;
    std::vector<void*> bufs;
    auto alloc = [&](size_t bytes, void** p) {
        const cudaError_t e = scratch_alloc(p, bytes, st);
        if (e == cudaSuccess) bufs.push_back(*p);
        return e;
    };
    auto done = [&](int rc, const std::string& msg) {
        for (void* p : bufs) cudaFreeAsync(p, st);
        const cudaError_t e = cudaStreamSynchronize(st);
        if (rc == GDBG_OK && e != cudaSuccess) return report_error(GDBG_ERR_CUDA, cudaGetErrorString(e));
        return rc == GDBG_OK ? rc : report_error(rc, msg);
    };
    // pass 1: newline counts per tile, their scan, the total and the last byte
    const uint64_t parts_t = scan32_partials_needed(n_tiles + 1) + 1;
    uint32_t *tile_cnt, *tile_base, *partials;
    uint64_t* info;
    cudaError_t e;
    if ((e = alloc((2 * n_tiles + parts_t) * sizeof(uint32_t), (void**)&tile_cnt)) != cudaSuccess ||
        (e = alloc(4 * sizeof(uint64_t), (void**)&info)) != cudaSuccess)
        return done(GDBG_ERR_OOM, std::string("parse scratch: ") + cudaGetErrorString(e));
    tile_base = tile_cnt + n_tiles;
    partials = tile_base + n_tiles;
    if (aligned) k_fx_count<true><<<(unsigned)n_tiles, FX_BLOCK, 0, st>>>(t, n_bytes, tile_cnt);
    else k_fx_count<false><<<(unsigned)n_tiles, FX_BLOCK, 0, st>>>(t, n_bytes, tile_cnt);
    if ((e = launch_scan32(tile_cnt, tile_base, n_tiles, partials, st)) != cudaSuccess)
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    uint32_t hb[2] = {0, 0};
    unsigned char edge[2] = {0, 0};
    cudaMemcpyAsync(&hb[0], tile_base + n_tiles - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hb[1], tile_cnt + n_tiles - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&edge[0], text, 1, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&edge[1], text + n_bytes - 1, 1, cudaMemcpyDeviceToHost, st);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (edge[0] != '>' && edge[0] != '@')
        return done(GDBG_ERR_UNSUPPORTED, "line 0: the text does not start with '>' or '@'; "
                                          "parse it on the host");
    const uint32_t n_nl = hb[0] + hb[1];
    const uint32_t n_lines = n_nl + (edge[1] != '\n' ? 1u : 0u);
    // pass 2: newline positions; per line the layout check, sequence bytes,
    // header flags; their scans
    const uint64_t parts_l = scan32_partials_needed((uint64_t)n_lines + 1) + 1;
    uint32_t *nlpos, *clen, *cpos, *hflag, *hidx, *lpart, *bad;
    if ((e = alloc(((uint64_t)n_nl + 4 * (uint64_t)n_lines + parts_l + 2) * sizeof(uint32_t),
                   (void**)&nlpos)) != cudaSuccess)
        return done(GDBG_ERR_OOM, std::string("parse scratch: ") + cudaGetErrorString(e));
    clen = nlpos + n_nl;
    cpos = clen + n_lines;
    hflag = cpos + n_lines;
    hidx = hflag + n_lines;
    lpart = hidx + n_lines;
    bad = lpart + parts_l;
    if ((e = cudaMemsetAsync(bad, 0xFF, 2 * sizeof(uint32_t), st)) != cudaSuccess)
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (aligned) k_fx_lines<true><<<(unsigned)n_tiles, FX_BLOCK, 0, st>>>(t, n_bytes, tile_base, nlpos, n_nl);
    else k_fx_lines<false><<<(unsigned)n_tiles, FX_BLOCK, 0, st>>>(t, n_bytes, tile_base, nlpos, n_nl);
    const unsigned lgrid = (unsigned)(((uint64_t)n_lines + FX_BLOCK - 1) / FX_BLOCK);
    k_fx_classify<<<lgrid, FX_BLOCK, 0, st>>>(t, n_bytes, nlpos, n_nl, n_lines, clen, hflag, bad,
                                              bad + 1);
    if ((e = launch_scan32(clen, cpos, n_lines, lpart, st)) != cudaSuccess ||
        (e = launch_scan32(hflag, hidx, n_lines, lpart, st)) != cudaSuccess)
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    k_fx_tail<<<1, 1, 0, st>>>(clen, cpos, hflag, hidx, n_lines, info);
    uint32_t hbad[2] = {0, 0};
    uint64_t hinfo[2] = {0, 0};
    cudaMemcpyAsync(hbad, bad, sizeof hbad, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hinfo, info, sizeof hinfo, cudaMemcpyDeviceToHost, st);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    if (hbad[0] != 0xFFFFFFFFu)
        return done(GDBG_ERR_UNSUPPORTED,
                    "line " + std::to_string(hbad[0]) + ": not a regular " +
                        (hbad[1] ? "FASTQ (four-line records)" : "FASTA") +
                        " layout; parse it on the host");
    const uint64_t seq_bytes = hinfo[0], n_rec = hinfo[1];
    stats[2] = n_rec;
    if (offsets_cap < n_rec + 1)
        return done(GDBG_ERR_INVALID_ARG, "offsets needs " + std::to_string(n_rec + 1) +
                                              " entries (the text's records + 1)");
    if (packed_words < seq_bytes / 16 + 1)
        return done(GDBG_ERR_INVALID_ARG, "packed needs " + std::to_string(seq_bytes / 16 + 1) + " words");
    // pass 3: the records' sequences -- FASTQ: spans of the text; FASTA:
    // their lines' bytes side by side -- then the packer
    const char* src;
    const uint64_t *starts, *ends;
    if (hbad[1]) {
        uint64_t* sp;
        if ((e = alloc(2 * n_rec * sizeof(uint64_t), (void**)&sp)) != cudaSuccess)
            return done(GDBG_ERR_OOM, std::string("parse scratch: ") + cudaGetErrorString(e));
        k_fx_spans<<<(unsigned)((n_rec + FX_BLOCK - 1) / FX_BLOCK), FX_BLOCK, 0, st>>>(
            t, n_bytes, nlpos, n_nl, n_rec, sp, sp + n_rec);
        src = text;
        starts = sp;
        ends = sp + n_rec;
    } else {
        unsigned char* seqs;
        uint64_t* so;
        if ((e = alloc(seq_bytes, (void**)&seqs)) != cudaSuccess ||
            (e = alloc((n_rec + 1) * sizeof(uint64_t), (void**)&so)) != cudaSuccess)
            return done(GDBG_ERR_OOM, std::string("parse scratch: ") + cudaGetErrorString(e));
        uint64_t ggrid = ((uint64_t)n_lines * 32 + FX_BLOCK - 1) / FX_BLOCK;
        if (ggrid > 152 * 32) ggrid = 152 * 32;
        k_fx_gather<<<(unsigned)ggrid, FX_BLOCK, 0, st>>>(t, n_bytes, nlpos, n_nl, n_lines, clen,
                                                          cpos, hflag, hidx, seqs, so);
        if ((e = cudaMemcpyAsync(so + n_rec, &hinfo[0], sizeof(uint64_t), cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
        src = (const char*)seqs;
        starts = so;
        ends = so + 1;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return done(GDBG_ERR_CUDA, cudaGetErrorString(e));
    uint64_t out[3];
    const int rc = pack_device_run(src, starts, ends, n_rec, min_length, packed, packed_words,
                                   offsets, out, st);
    if (rc != GDBG_OK) {
        for (void* p : bufs) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        return rc;
    }
    stats[0] = out[0];
    stats[1] = out[1];
    stats[3] = out[1] + out[2];
    return done(GDBG_OK, "");
}
