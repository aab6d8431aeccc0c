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
