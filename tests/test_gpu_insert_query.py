"""Order-exact insert_and_query on the GPU (gdbg_insert_and_query_batch and
the per-read gdbg_insert_and_query_sequence): every k-mer's count equals what
dBG::insert_and_query_sequence returns when the reads are inserted one after
another (dbg.hh:327-340; bytestorage.cc:142-150, nibblestorage.cc:103-109,
bitstorage.cc:78-84), against the reference's golden counts and the oracle."""
import numpy as np
import pytest

import oracle
from goldens import Case, names
import goetia_gb300 as G
from goetia_gb300 import synth
from goetia_gb300.reads import PackedReads

pytestmark = pytest.mark.gpu

STORAGES = {"bit": G.BitStorage, "byte": G.ByteStorage, "nibble": G.NibbleStorage}
SHIFTERS = {True: G.CanLemireShifter, False: G.FwdLemireShifter}


def graph_for(kind, canonical, K, sizes):
    st = STORAGES[kind](tablesizes=[int(s) for s in sizes])
    return G.dBG[STORAGES[kind], SHIFTERS[canonical]].build(st, K)


@pytest.mark.parametrize("bucket_bits", [0, 5, 7])
@pytest.mark.parametrize("name", names())
def test_golden_batch(cuda_ready, name, bucket_bits):
    c = Case(name)
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    if bucket_bits:
        g.set_bucket_bits(bucket_bits)
    packed, off = c.packed()
    counts, n_new = g.insert_and_query_packed(PackedReads(packed, off))
    assert np.array_equal(counts, c.iq_counts)
    assert np.array_equal(n_new, c.n_new)
    for a, b in zip(g.get_raw(), c.tables):
        assert np.array_equal(a, b)
    assert (g.n_unique(), g.n_occupied()) == (c.n_unique, c.n_occupied)


@pytest.mark.parametrize("name", names())
def test_golden_per_read(cuda_ready, name):
    c = Case(name)
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    got = []
    for s in c.reads:
        if len(s) < c.K:
            with pytest.raises(G.SequenceLengthException):
                g.insert_and_query_sequence(s)
            continue
        got += g.insert_and_query_sequence(s)
    assert got == [int(x) for x in c.iq_counts]
    # the hashes+counts overload of insert_sequence on a fresh graph
    h = graph_for(c.storage, c.canonical, c.K, c.sizes)
    hashes, counts = [], []
    for s in c.reads:
        if len(s) >= c.K:
            h.insert_sequence(s, hashes, counts)
    assert counts == [int(x) for x in c.iq_counts]
    assert [int(x) for x in hashes] == [int(x) for x in c.val]


@pytest.mark.parametrize("kind", ["byte", "nibble"])
def test_high_coverage_against_oracle(cuda_ready, kind):
    """High coverage (many repeats of each k-mer within a batch, counts that
    saturate) on tables of ~2^24 cells, in three consecutive batches."""
    sizes = oracle.primes(4, 1 << 24)
    g = graph_for(kind, True, 31, sizes)
    ref = oracle.Storage(kind, sizes)
    gen = synth.genome(200_000, 21)
    for b in range(3):
        rows = synth.sample_reads(gen, 40_000, 150, 0.002, 100 + b)
        pr = synth.rows_to_packed(rows)
        counts, n_new = g.insert_and_query_packed(pr)
        want = ref.insert_and_query_reads(True, 31, pr.packed, pr.offsets)
        assert np.array_equal(counts, want), b
    for a, t in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, t)
    assert g.n_occupied() == ref.stats()[1]


def test_device_entry_point(cuda_ready):
    import torch
    c = Case("nibble_fwd_k21")
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    packed, off = c.packed()
    dp = torch.from_numpy(packed.view(np.int32)).cuda()
    do = torch.from_numpy(off.view(np.int64)).cuda()
    n = int(c.iq_counts.size)
    counts = torch.zeros(n, dtype=torch.int16, device="cuda")
    n_new = torch.zeros(len(off) - 1, dtype=torch.int64, device="cuda")
    g.insert_and_query_device(dp.data_ptr(), dp.numel(), do.data_ptr(), len(off) - 1,
                              counts.data_ptr(), n_new.data_ptr(), stream=0)
    torch.cuda.synchronize()
    assert np.array_equal(counts.cpu().numpy(), c.iq_counts)
    assert np.array_equal(n_new.cpu().numpy().view(np.uint64), c.n_new)
