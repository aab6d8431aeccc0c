"""Batched uneven-length insert (config 3 shape, scaled down): fixed-capacity
batches replayed through a CUDA graph, and the autotuner, against the oracle's
sequential insert."""
import numpy as np
import pytest

import oracle
import goetia_gb300 as G
from goetia_gb300 import batched, synth

pytestmark = pytest.mark.gpu


def _reads(seed=10, n=400):
    gens = [synth.genome(200_000, 5 + i) for i in range(5)]
    return synth.uneven_batch(gens, [1, 2, 4, 8, 16], n, 1500, 1.0, 200, 20000, 0.04, 0.02,
                              0.02, seed)


@pytest.mark.parametrize("use_graph", [True, False])
def test_batched_uneven_vs_oracle(cuda_ready, use_graph):
    pr = _reads()
    sizes = oracle.primes(4, 1 << 21)
    ref = oracle.Storage("nibble", sizes)
    _, want = ref.insert_reads(False, 21, pr.packed, pr.offsets)
    g = G.dBG[G.NibbleStorage, G.FwdLemireShifter].build(G.NibbleStorage(tablesizes=sizes), 21)
    g.set_bucket_bits(12)
    ins = batched.BatchedInserter(g, max_reads=96, max_bases=200_000, use_graph=use_graph)
    ins.prepare()
    assert (ins.cuda_graph is not None) == use_graph
    got = ins.insert_stream(pr)
    assert np.array_equal(got, want)
    for a, b in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, b)
    assert (g.n_unique(), g.n_occupied()) == ref.stats()


def test_persistent_kernel_graph_replay_vs_oracle(cuda_ready):
    """The persistent fused hash+insert kernel captured once in a CUDA graph
    and replayed per batch: per-read new counts, tables and counters equal
    the oracle's sequential insert."""
    pr = _reads(seed=12)
    sizes = oracle.primes(4, 1 << 21)
    ref = oracle.Storage("nibble", sizes)
    _, want = ref.insert_reads(False, 21, pr.packed, pr.offsets)
    g = G.dBG[G.NibbleStorage, G.FwdLemireShifter].build(G.NibbleStorage(tablesizes=sizes), 21)
    g.set_insert_path("persistent")
    g.set_insert_schedule(65536, 4)
    ins = batched.BatchedInserter(g, max_reads=96, max_bases=200_000, use_graph=True).prepare()
    assert ins.cuda_graph is not None and g.insert_path() == "persistent"
    assert np.array_equal(ins.insert_stream(pr), want)
    for a, b in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, b)
    assert (g.n_unique(), g.n_occupied()) == ref.stats()


def test_autotune_then_insert(cuda_ready, tmp_path, monkeypatch):
    monkeypatch.setenv("GOETIA_GB300_CACHE", str(tmp_path))
    pr = _reads(seed=11, n=200)
    sizes = oracle.primes(4, 1 << 22)
    g = G.dBG[G.NibbleStorage, G.FwdLemireShifter].build(G.NibbleStorage(tablesizes=sizes), 21)
    batches = batched.split_batches(pr, 64, 150_000)
    best = batched.autotune(g, batches[0][1], 64, 150_000)
    assert best["schedule"]["path"] in ("bucketed", "bucketed_ordered", "persistent")
    assert {t["schedule"]["path"] for t in best["trials"]} >= {"bucketed", "persistent"}
    again = batched.autotune(g, batches[0][1], 64, 150_000)   # from the cache
    assert again["schedule"] == best["schedule"]
    ref = oracle.Storage("nibble", sizes)
    _, want = ref.insert_reads(False, 21, pr.packed, pr.offsets)
    ins = batched.BatchedInserter(g, 64, 150_000).prepare()
    assert np.array_equal(ins.insert_stream(pr), want)
