"""The segmented insert's apply on crowded buckets, against the oracle.

The apply stages a bucket's records in shared memory and keys every cell
that was zero before the batch to its first toucher (the record with the
smallest k-mer ordinal) in a map.  Ordinary batches take one pass; these
cases force the other paths by fixing large buckets on small tables:

* all of a bucket's records staged, but more zero cells than the map
  holds (a fresh, empty table): the cells are taken in narrower ranges;
* more records than the staging buffer holds: records are staged in
  chunks, per cell range.

Each must give the sequential insert's per-read new counts, table bytes and
counters (bitstorage.hh:195-219, bytestorage.cc:60-113, nibblestorage.cc:
60-100), over two batches (empty tables, then a mix of seen and fresh cells).
"""
import numpy as np
import pytest

import oracle
import goetia_gb300 as G
from goetia_gb300 import synth

pytestmark = pytest.mark.gpu

STORAGES = {"bit": G.BitStorage, "byte": G.ByteStorage, "nibble": G.NibbleStorage}


@pytest.mark.parametrize("kind,bucket_bits,n_reads", [
    ("nibble", 14, 14_000),   # ~6,500 records per bucket: one chunk, narrowed cell ranges
    ("byte", 14, 28_000),     # ~13,000 records per bucket: two chunks
    ("bit", 15, 24_000),      # ~22,500 records per bucket: three chunks
])
def test_crowded_buckets_match_oracle(cuda_ready, kind, bucket_bits, n_reads):
    sizes = oracle.primes(4, 1 << 22)
    st = STORAGES[kind]
    g = G.dBG[st, G.CanLemireShifter].build(st(tablesizes=sizes), 31)
    g.set_insert_path("bucketed")
    g.set_bucket_bits(bucket_bits)
    g.set_profiling(True)
    ref = oracle.Storage(kind, sizes)
    gen = synth.genome(3_000_000, 61)
    for b in range(2):
        pr = synth.rows_to_packed(synth.sample_reads(gen, n_reads, 150, 0.01, 62 + b))
        got = g.insert_packed(pr)
        _, want = ref.insert_reads(True, 31, pr.packed, pr.offsets)
        assert np.array_equal(got, want), b
    assert "k_sp_apply" in g.stage_times()
    assert (g.n_unique(), g.n_occupied()) == ref.stats()
    for a, w in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, w)
