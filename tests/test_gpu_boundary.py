"""The segmented insert at the edge of its 32-bit cell-id space.

The segmented bucketed path numbers every cell of every table in one global
space, each table padded up to whole buckets, and packs each record as
(global cell << 32) | k-mer ordinal.  Four tables just below 2^30 cells pad
to exactly 2^30 each, so the padded space is exactly 2^32 and the last
bucket of table 3 ends at cell id 0xFFFFFFFF: the headline ByteStorage
workload (4 x ~2^30 cells) sits on this boundary.  Bit tables of the same
cell counts (512 MiB) reach the same ids in far less memory.  The insert
must equal the oracle's sequential insert (bitstorage.hh:195-219,
bytestorage.cc:60-113): per-read new counts, n_unique / n_occupied, and the
table bytes, including the k-mers that land in the last bucket.
"""
import numpy as np
import pytest

import oracle
import goetia_gb300 as G
from goetia_gb300 import synth

pytestmark = pytest.mark.gpu

BIT_BUCKET_CELLS = 1 << 18    # 32 KB of Bit table per bucket (the segmented default)


def test_bit_tables_padded_to_exactly_2_32_cells(cuda_ready):
    sizes = oracle.primes(4, 1 << 30)
    padded = sum((p + BIT_BUCKET_CELLS - 1) // BIT_BUCKET_CELLS * BIT_BUCKET_CELLS for p in sizes)
    assert padded == 1 << 32
    gen = synth.genome(3_000_000, 91)
    batches = [synth.rows_to_packed(synth.sample_reads(gen, 60_000, 150, 0.01, 92 + i))
               for i in range(2)]
    g = G.dBG[G.BitStorage, G.CanLemireShifter].build(G.BitStorage(tablesizes=sizes), 31)
    g.set_insert_path("bucketed")
    g.set_profiling(True)
    ref = oracle.Storage("bit", sizes)
    last_bucket_hits = 0
    for pr in batches:
        got = g.insert_packed(pr)
        _, want = ref.insert_reads(True, 31, pr.packed, pr.offsets)
        assert np.array_equal(got, want)
        vals, _, _ = oracle.hash_reads(True, 31, pr.packed, pr.offsets)
        p3 = np.uint64(sizes[3])
        last_bucket_hits += int(((vals % p3) >= p3 - np.uint64(BIT_BUCKET_CELLS)).sum())
    assert "k_sp_apply" in g.stage_times()   # the segmented path ran
    assert last_bucket_hits > 0
    assert (g.n_unique(), g.n_occupied()) == ref.stats()
    for a, b in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, b)
