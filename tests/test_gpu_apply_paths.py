"""The segmented insert's apply on crowded buckets, against the oracle.

The apply reads a bucket's records once: cells that were not zero before
the batch take their increments at once, zero cells are counted in a
shared-memory map that keeps each one's first toucher (the record with the
smallest k-mer ordinal) and get their values after the last record.
Ordinary batches fit the map; these cases force the other paths by fixing
large buckets on small tables:

* fresh, empty tables with more zero cells per bucket than the map holds:
  the zero cells are redone in narrower cell ranges, the increments stand;
* a small genome read many times over: hundreds of touches per cell in one
  batch, so counts saturate (255 / 15) on cells that were zero before it;
* one read repeated: the records crowd a few digit groups and buckets far
  past their reserved slots, so both partition passes fall back to their
  counted layouts.

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


@pytest.mark.parametrize("kind,bucket_bits,n_reads,genome_bp", [
    ("nibble", 14, 14_000, 3_000_000),   # ~6,500 records, ~5,400 zero cells per bucket
    ("byte", 15, 28_000, 3_000_000),     # ~26,000 records, ~18,000 zero cells: ranges
    ("bit", 15, 24_000, 3_000_000),      # ~22,500 records, ~16,000 zero cells: ranges
    ("byte", 15, 20_000, 2_000),         # ~600 touches per k-mer in each batch
    ("nibble", 14, 20_000, 2_000),
    ("byte", 15, 20_000, 150),           # one read, 20,000 times: every group and bucket
                                         # but a few empty, the rest far over their slots
])
def test_crowded_buckets_match_oracle(cuda_ready, kind, bucket_bits, n_reads, genome_bp):
    sizes = oracle.primes(4, 1 << 22)
    st = STORAGES[kind]
    g = G.dBG[st, G.CanLemireShifter].build(st(tablesizes=sizes), 31)
    g.set_insert_path("bucketed")
    g.set_bucket_bits(bucket_bits)
    g.set_profiling(True)
    ref = oracle.Storage(kind, sizes)
    gen = synth.genome(genome_bp, 61)
    for b in range(2):
        pr = synth.rows_to_packed(synth.sample_reads(gen, n_reads, 150, 0.01, 62 + b))
        got = g.insert_packed(pr)
        _, want = ref.insert_reads(True, 31, pr.packed, pr.offsets)
        assert np.array_equal(got, want), b
    assert "k_sp_apply" in g.stage_times()
    assert (g.n_unique(), g.n_occupied()) == ref.stats()
    for a, w in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, w)
