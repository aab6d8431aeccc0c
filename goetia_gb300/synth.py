"""Seeded synthetic genomes and reads (numpy), shared by the tests and bench.

No public dataset is involved anywhere: every workload is generated here
from fixed seeds with the shapes of the benchmark configurations (uniform
random ACGT genomes; reads sampled uniformly from either strand with i.i.d.
errors).  Codes are A=0 C=1 G=2 T=3.
"""
import numpy as np

from .reads import PackedReads, pack_codes


def genome(n, seed):
    return np.random.default_rng(seed).integers(0, 4, n, dtype=np.uint8)


def revcomp(codes):
    return (3 - codes[..., ::-1]).astype(np.uint8)


def substitute(rows, rate, rng):
    """i.i.d. substitutions to a different base, in place on a 2-D code array."""
    n = rows.size
    k = rng.binomial(n, rate)
    if k:
        idx = rng.integers(0, n, k)
        flat = rows.reshape(-1)
        flat[idx] = (flat[idx] + rng.integers(1, 4, k, dtype=np.uint8)) & 3
    return rows


def sample_reads(g, n_reads, length, sub_rate, seed, rc_frac=0.5):
    """n_reads x length code array: uniform starts, strand flip, substitutions."""
    rng = np.random.default_rng(seed)
    starts = rng.integers(0, len(g) - length + 1, n_reads)
    win = np.lib.stride_tricks.sliding_window_view(g, length)
    rows = win[starts].copy()
    flip = rng.random(n_reads) < rc_frac
    if flip.any():
        rows[flip] = 3 - rows[flip][:, ::-1]
    substitute(rows, sub_rate, rng)
    return rows


def pack_codes_np(codes):
    """uint8 codes (A=0 C=1 G=2 T=3) -> uint32 packed stream in numpy alone
    (the same words as reads.pack_codes: base j in bits 2*(j%16) of word
    j/16, len(codes)//16 + 1 words, zero-padded).  Four codes make a byte,
    four bytes a little-endian word."""
    codes = np.ascontiguousarray(codes, np.uint8)
    n = len(codes)
    buf = np.zeros((n // 16 + 1) * 16, np.uint8)
    buf[:n] = codes
    q = buf.reshape(-1, 4)
    b = q[:, 0] | (q[:, 1] << 2) | (q[:, 2] << 4) | (q[:, 3] << 6)
    return b.view("<u4").astype(np.uint32, copy=False)


def rows_to_packed(rows, native=True):
    """Equal-length code rows -> PackedReads.  native=False packs with numpy
    alone, so the caller never loads the GPU library."""
    rows = np.ascontiguousarray(rows, np.uint8)
    n, L = rows.shape
    offsets = np.arange(n + 1, dtype=np.uint64) * np.uint64(L)
    flat = rows.reshape(-1)
    return PackedReads(pack_codes(flat) if native else pack_codes_np(flat), offsets, 0)


def n_read_mask(n_reads, frac, seed):
    """Reads that carry an 'N' (dropped by the FASTX policy before packing)."""
    return np.random.default_rng(seed).random(n_reads) < frac


def uneven_reads(genomes, abundances, n_reads, median, sigma, lo, hi, sub, ins, dele, seed):
    """Log-normal read lengths from several genomes with indel errors.

    Returns a list of code arrays.  Each read is drawn from genome i with
    probability proportional to abundances[i]; errors are applied per base:
    substitution (to a different base), insertion (a random base before it)
    or deletion, with the given rates.
    """
    rng = np.random.default_rng(seed)
    w = np.asarray(abundances, float)
    src = rng.choice(len(genomes), n_reads, p=w / w.sum())
    lens = np.clip(np.exp(rng.normal(np.log(median), sigma, n_reads)), lo, hi).astype(np.int64)
    out = []
    for i in range(n_reads):
        g = genomes[src[i]]
        L = int(min(lens[i], len(g)))
        s = int(rng.integers(0, len(g) - L + 1))
        r = g[s:s + L].copy()
        if rng.random() < 0.5:
            r = revcomp(r)
        u = rng.random(L)
        keep = u >= dele
        subm = (u >= dele) & (u < dele + sub)
        r[subm] = (r[subm] + rng.integers(1, 4, int(subm.sum()), dtype=np.uint8)) & 3
        insm = (u >= dele + sub) & (u < dele + sub + ins)
        pieces = []
        ins_pos = np.nonzero(insm)[0]
        prev = 0
        for p in ins_pos:
            pieces.append(r[prev:p][keep[prev:p]])
            pieces.append(rng.integers(0, 4, 1, dtype=np.uint8))
            prev = p
        pieces.append(r[prev:][keep[prev:]])
        out.append(np.concatenate(pieces).astype(np.uint8))
    return out


def list_to_packed(reads):
    flat = np.concatenate(reads) if reads else np.zeros(0, np.uint8)
    offsets = np.zeros(len(reads) + 1, np.uint64)
    if reads:
        offsets[1:] = np.cumsum([len(r) for r in reads], dtype=np.uint64)
    return PackedReads(pack_codes(flat), offsets, 0)


def uneven_batch(genomes, abundances, n_reads, median, sigma, lo, hi, sub, ins, dele, seed):
    """Vectorised uneven_reads: returns PackedReads directly.

    Read lengths are log-normal (median, sigma) clipped to [lo, hi]; each read
    comes from genome i with probability proportional to abundances[i], from
    either strand; every base is independently deleted (dele), substituted
    (sub) or followed by an inserted random base (ins)."""
    rng = np.random.default_rng(seed)
    w = np.asarray(abundances, float)
    src = rng.choice(len(genomes), n_reads, p=w / w.sum())
    lens = np.clip(np.exp(rng.normal(np.log(median), sigma, n_reads)), lo, hi).astype(np.int64)
    glen = np.array([len(g) for g in genomes], np.int64)
    lens = np.minimum(lens, glen[src])
    starts = (rng.random(n_reads) * (glen[src] - lens + 1)).astype(np.int64)
    cat = np.concatenate(genomes)
    gbase = np.concatenate([[0], np.cumsum(glen)[:-1]])
    total = int(lens.sum())
    read_of = np.repeat(np.arange(n_reads), lens)
    pos_in = np.arange(total) - np.repeat(np.cumsum(lens) - lens, lens)
    flip = rng.random(n_reads) < 0.5
    fr = flip[read_of]
    src_pos = gbase[src][read_of] + starts[read_of] + np.where(fr, lens[read_of] - 1 - pos_in, pos_in)
    bases = cat[src_pos]
    bases = np.where(fr, 3 - bases, bases).astype(np.uint8)
    u = rng.random(total, dtype=np.float32)
    subm = (u >= dele) & (u < dele + sub)
    bases[subm] = (bases[subm] + rng.integers(1, 4, int(subm.sum()), dtype=np.uint8)) & 3
    reps = np.where(u < dele, 0, np.where(u < dele + sub + ins, np.where(u >= dele + sub, 2, 1), 1))
    out = np.repeat(bases, reps)
    # the second copy of each inserted base becomes a random base
    ins_at = np.cumsum(reps)[reps == 2] - 1
    out[ins_at] = rng.integers(0, 4, len(ins_at), dtype=np.uint8)
    new_lens = np.add.reduceat(reps, np.cumsum(lens) - lens) if n_reads else np.zeros(0, np.int64)
    new_lens = np.where(lens > 0, new_lens, 0)
    offsets = np.zeros(n_reads + 1, np.uint64)
    offsets[1:] = np.cumsum(new_lens, dtype=np.uint64)
    return PackedReads(pack_codes(out), offsets, 0)


def repeat_genome(n, n_repeats, rep_lo, rep_hi, snp_rate, seed):
    """A genome with inserted repeats plus a SNP haplotype (decision-node
    workload): n random bases, n_repeats copies of random 1-5 kb segments
    pasted at random positions, and a second haplotype with i.i.d. SNPs at
    snp_rate.  Returns (haplotype_a, haplotype_b) as code arrays."""
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 4, n, dtype=np.uint8)
    for _ in range(n_repeats):
        L = int(rng.integers(rep_lo, rep_hi + 1))
        src = int(rng.integers(0, n - L))
        dst = int(rng.integers(0, n - L))
        g[dst:dst + L] = g[src:src + L].copy()
    h = g.copy()
    k = rng.binomial(n, snp_rate)
    idx = rng.integers(0, n, k)
    h[idx] = (h[idx] + rng.integers(1, 4, k, dtype=np.uint8)) & 3
    return g, h


def tiles_of(seq, tile, K):
    """Cut a long sequence into reads of `tile` bases overlapping by K-1, so
    every k-mer of seq is in exactly one read."""
    step = tile - (K - 1)
    starts = np.arange(0, max(len(seq) - K + 1, 1), step)
    reads = [seq[s:s + tile] for s in starts]
    return list_to_packed(reads)


# ---- multi-threaded generator (goetia_gb300/workload/gen_reads.cc) ---------
#
# Every random choice of these generators is a pure function of (seed, read,
# position): a splitmix64-style mix, restated below in numpy (the *_np twins,
# used by the tests on small cases to pin the C++ generator bit for bit).

_WL = None
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _wl():
    global _WL
    if _WL is None:
        import ctypes
        from . import build as _build
        path = _build.build_workload()
        L = ctypes.CDLL(path)
        u8p, u32p, u64p = (ctypes.POINTER(t) for t in (ctypes.c_uint8, ctypes.c_uint32,
                                                          ctypes.c_uint64))
        L.wl_sample_reads.argtypes = [u8p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_uint64, ctypes.c_double, ctypes.c_uint64, u32p, u64p,
                                      ctypes.c_int]
        common = [u8p, u64p, ctypes.c_uint32, u32p, u64p, u32p, u8p, ctypes.c_uint64,
                  ctypes.c_uint64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_uint64]
        L.wl_uneven_lengths.argtypes = common + [u64p, ctypes.c_int]
        L.wl_uneven_write.argtypes = common + [u64p, u32p, ctypes.c_int]
        for f in (L.wl_sample_reads, L.wl_uneven_lengths, L.wl_uneven_write):
            f.restype = ctypes.c_int
        _WL = (L, u8p, u32p, u64p)
    return _WL


def _threads(threads):
    import os
    return int(threads or os.cpu_count() or 1)


def sample_reads_packed(g, n_reads, length, sub_rate, seed, first_read=0, threads=None):
    """n_reads reads of `length` bases from genome g as PackedReads, made by
    the C++ generator: uniform start, either strand, i.i.d. substitutions
    (reads first_read .. first_read + n_reads - 1 of the seed's stream)."""
    L, u8p, u32p, u64p = _wl()
    g = np.ascontiguousarray(g, np.uint8)
    packed = np.zeros(n_reads * length // 16 + 1, np.uint32)
    offsets = np.zeros(n_reads + 1, np.uint64)
    rc = L.wl_sample_reads(g.ctypes.data_as(u8p), len(g), n_reads, length, seed, sub_rate,
                           first_read, packed.ctypes.data_as(u32p), offsets.ctypes.data_as(u64p),
                           _threads(threads))
    if rc:
        raise ValueError("wl_sample_reads: bad arguments")
    return PackedReads(packed, offsets, 0)


def uneven_plan(genome_lens, abundances, n_reads, median, sigma, lo, hi, seed):
    """Per-read source windows of the uneven workload (numpy, seeded): genome
    drawn by abundance, log-normal length (median, sigma) clipped to [lo, hi]
    and to the genome, uniform start, strand 50/50."""
    rng = np.random.default_rng(seed)
    w = np.asarray(abundances, float)
    src = rng.choice(len(genome_lens), n_reads, p=w / w.sum()).astype(np.uint32)
    lens = np.clip(np.exp(rng.normal(np.log(median), sigma, n_reads)), lo, hi).astype(np.int64)
    glen = np.asarray(genome_lens, np.int64)
    lens = np.minimum(lens, glen[src])
    starts = (rng.random(n_reads) * (glen[src] - lens + 1)).astype(np.uint64)
    flip = (rng.random(n_reads) < 0.5).astype(np.uint8)
    return src, starts, lens.astype(np.uint32), flip


def uneven_stream(genomes, abundances, n_reads, median, sigma, lo, hi, sub, ins, dele, seed,
                  threads=None):
    """The uneven-length workload as one PackedReads, made by the C++
    generator: uneven_plan's windows, then per source base a deletion,
    substitution or an inserted random base after it, at the given rates."""
    L, u8p, u32p, u64p = _wl()
    cat = np.ascontiguousarray(np.concatenate(genomes), np.uint8)
    goff = np.zeros(len(genomes) + 1, np.uint64)
    goff[1:] = np.cumsum([len(x) for x in genomes])
    src, starts, lens, flip = uneven_plan([len(x) for x in genomes], abundances, n_reads, median,
                                          sigma, lo, hi, seed)
    args = [cat.ctypes.data_as(u8p), goff.ctypes.data_as(u64p), len(genomes),
            src.ctypes.data_as(u32p), starts.ctypes.data_as(u64p), lens.ctypes.data_as(u32p),
            flip.ctypes.data_as(u8p), n_reads, seed, sub, ins, dele, 0]
    out_len = np.zeros(max(n_reads, 1), np.uint64)
    if L.wl_uneven_lengths(*args, out_len.ctypes.data_as(u64p), _threads(threads)):
        raise ValueError("wl_uneven_lengths: bad arguments")
    offsets = np.zeros(n_reads + 1, np.uint64)
    offsets[1:] = np.cumsum(out_len[:n_reads], dtype=np.uint64)
    packed = np.zeros(int(offsets[-1]) // 16 + 1, np.uint32)
    if L.wl_uneven_write(*args, offsets.ctypes.data_as(u64p), packed.ctypes.data_as(u32p),
                         _threads(threads)):
        raise ValueError("wl_uneven_write: bad arguments")
    return PackedReads(packed, offsets, 0)


def _mix_np(z):
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _key_np(seed, read):
    with np.errstate(over="ignore"):
        return np.uint64(seed) ^ _mix_np(np.uint64(read) + np.uint64(0x9E3779B97F4A7C15))


def _draw_np(key, pos):
    with np.errstate(over="ignore"):
        return _mix_np(key ^ (np.asarray(pos, np.uint64) * np.uint64(0xD6E8FEB86659FD93)))


def _threshold(rate):
    return int(min(max(rate * (1 << 24), 0.0), float(1 << 24)) + 0.5)


def sample_reads_packed_np(g, n_reads, length, sub_rate, seed, first_read=0):
    """numpy twin of sample_reads_packed (small cases)."""
    ts = _threshold(sub_rate)
    span = len(g) - length + 1
    rows = np.zeros((n_reads, length), np.uint8)
    j = np.arange(length, dtype=np.uint64)
    for r in range(n_reads):
        key = _key_np(seed, first_read + r)
        start = int(_draw_np(key, 1 << 40) % np.uint64(span))
        flip = bool(_draw_np(key, (1 << 40) + 1) >> np.uint64(63))
        b = g[start:start + length].astype(np.uint8)
        if flip:
            b = (3 - b[::-1]).astype(np.uint8)
        x = _draw_np(key, j)
        s = (x >> np.uint64(40)) < np.uint64(ts)
        off = (np.uint64(1) + (x >> np.uint64(8)) % np.uint64(3)).astype(np.uint8)
        rows[r] = np.where(s, (b + off) & 3, b)
    return rows_to_packed(rows, native=False)


def uneven_stream_np(genomes, abundances, n_reads, median, sigma, lo, hi, sub, ins, dele, seed):
    """numpy twin of uneven_stream (small cases)."""
    src, starts, lens, flip = uneven_plan([len(x) for x in genomes], abundances, n_reads, median,
                                          sigma, lo, hi, seed)
    td, tsd, tisd = _threshold(dele), _threshold(dele + sub), _threshold(dele + sub + ins)
    out = []
    for r in range(n_reads):
        g = genomes[int(src[r])]
        L, s0 = int(lens[r]), int(starts[r])
        b = g[s0:s0 + L].astype(np.uint8)
        if flip[r]:
            b = (3 - b[::-1]).astype(np.uint8)
        key = _key_np(seed, r)
        x = _draw_np(key, np.arange(L, dtype=np.uint64))
        u = (x >> np.uint64(40)).astype(np.int64)
        off = (np.uint64(1) + (x >> np.uint64(8)) % np.uint64(3)).astype(np.uint8)
        b = np.where((u >= td) & (u < tsd), (b + off) & 3, b).astype(np.uint8)
        ins_b = ((x >> np.uint64(16)) & np.uint64(3)).astype(np.uint8)
        pieces = []
        for j in range(L):
            if u[j] < td:
                continue
            pieces.append(b[j])
            if tsd <= u[j] < tisd:
                pieces.append(ins_b[j])
        out.append(np.array(pieces, np.uint8))
    flat = np.concatenate(out) if out else np.zeros(0, np.uint8)
    offsets = np.zeros(n_reads + 1, np.uint64)
    offsets[1:] = np.cumsum([len(o) for o in out])
    return PackedReads(pack_codes_np(flat), offsets, 0)
