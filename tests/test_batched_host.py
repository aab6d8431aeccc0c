"""Host-side batch splitting for the batched inserter (no GPU)."""
import numpy as np

from goetia_gb300 import batched, synth


def test_split_batches_respects_capacity_and_covers_reads():
    gens = [synth.genome(50_000, 1)]
    pr = synth.uneven_batch(gens, [1], 300, 800, 1.0, 50, 5000, 0.01, 0.0, 0.0, 3)
    parts = batched.split_batches(pr, 37, 20_000)
    r = 0
    j = np.arange(int(pr.offsets[-1]))
    codes = (pr.packed[j >> 4] >> (2 * (j & 15)).astype(np.uint32)) & 3
    for r0, b in parts:
        assert r0 == r
        assert b.n_reads <= 37 and b.n_bases <= 20_000
        for k in range(b.n_reads):
            a0, a1 = int(b.offsets[k]), int(b.offsets[k + 1])
            jj = np.arange(a0, a1)
            got = (b.packed[jj >> 4] >> (2 * (jj & 15)).astype(np.uint32)) & 3
            s0, s1 = int(pr.offsets[r + k]), int(pr.offsets[r + k + 1])
            assert np.array_equal(got, codes[s0:s1])
        r += b.n_reads
    assert r == pr.n_reads


def test_concat_keeps_every_read():
    from goetia_gb300.reads import concat
    gens = [synth.genome(80_000, 2)]
    parts = [synth.uneven_batch(gens, [1], 40, 300, 1.0, 30, 2000, 0.04, 0.02, 0.02, s)
             for s in (4, 5, 6)]
    c = concat(parts)

    def codes(p):
        j = np.arange(int(p.offsets[-1]))
        return (p.packed[j >> 4] >> (2 * (j & 15)).astype(np.uint32)) & 3

    cc, r = codes(c), 0
    for p in parts:
        cp = codes(p)
        for k in range(p.n_reads):
            assert np.array_equal(cp[int(p.offsets[k]):int(p.offsets[k + 1])],
                                  cc[int(c.offsets[r]):int(c.offsets[r + 1])])
            r += 1
    assert r == c.n_reads
