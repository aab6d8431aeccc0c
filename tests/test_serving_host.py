"""Host-side logic of the serving loop (no GPU): workload generation and
HBM footprint accounting."""
import numpy as np

import goetia_gb300 as G
from goetia_gb300 import serving


def test_make_streams_is_seeded_and_ordered():
    a = serving.make_streams(4, 11, 100, 1000, 8, 256, 16, 18, 0.001, genome_len=50_000)
    b = serving.make_streams(4, 11, 100, 1000, 8, 256, 16, 18, 0.001, genome_len=50_000)
    for x, y in zip(a, b):
        assert x.max_table == y.max_table and x.arrivals == y.arrivals
        assert all(np.array_equal(c.packed, d.packed) for c, d in zip(x.chunks, y.chunks))
        assert all(t1 <= t2 for t1, t2 in zip(x.arrivals, x.arrivals[1:]))
        assert all(8 <= c.n_reads <= 256 for c in x.chunks[:-1])
        assert 100 <= sum(c.n_reads for c in x.chunks) <= 1000


def test_footprint_grows_with_tables():
    small = serving.stream_footprint(G.BitStorage, 1 << 16, 4, 65536)
    large = serving.stream_footprint(G.BitStorage, 1 << 24, 4, 65536)
    assert large - small >= 4 * ((1 << 24) - (1 << 16)) // 8 - 4 * 256
