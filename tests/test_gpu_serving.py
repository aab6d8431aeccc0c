"""Serving loop (config 5 shape, scaled down): continuous batching over many
streams gives every chunk the same per-read new-k-mer counts as a sequential
replay of its stream, alone or in the mix, under HBM-budget admission."""
import numpy as np
import pytest

import goetia_gb300 as G
from goetia_gb300 import serving

pytestmark = pytest.mark.gpu


def _specs(seed=3, n=8):
    return serving.make_streams(n, seed, reads_lo=200, reads_hi=3000, chunk_lo=8, chunk_hi=512,
                                table_lo_bits=16, table_hi_bits=20, mean_gap_s=0.002,
                                genome_len=200_000)


def _check_exact(specs, results):
    for spec in specs:
        want = serving.replay(spec)
        got = results[spec.sid]
        assert [r.index for r in got] == list(range(len(spec.chunks)))
        for r, w in zip(got, want):
            assert np.array_equal(r.n_new, w), (spec.sid, r.index)


def test_serving_matches_sequential_replay(cuda_ready):
    specs = _specs()
    srv = serving.Server(G.BitStorage, G.CanLemireShifter, K=31, hbm_budget=8 << 30, depth=3)
    results, stats = srv.run(specs)
    assert stats["chunks"] == sum(len(s.chunks) for s in specs)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    _check_exact(specs, results)


def test_stream_alone_equals_stream_in_mix(cuda_ready):
    specs = _specs(seed=5)
    srv = serving.Server(G.BitStorage, G.CanLemireShifter, K=31, hbm_budget=8 << 30)
    mixed, _ = srv.run(specs)
    alone, _ = srv.run([specs[2]])
    for a, b in zip(alone[specs[2].sid], mixed[specs[2].sid]):
        assert np.array_equal(a.n_new, b.n_new)


def test_admission_by_hbm_budget(cuda_ready):
    specs = serving.make_streams(6, 7, reads_lo=1000, reads_hi=3000, chunk_lo=8, chunk_hi=256,
                                 table_lo_bits=16, table_hi_bits=20, mean_gap_s=0.002,
                                 genome_len=200_000, start_spread_s=0.001)
    srv = serving.Server(G.BitStorage, G.CanLemireShifter, K=31, window=65536)
    need = sorted(srv.footprint(s) for s in specs)
    srv.budget = need[-1] + need[-2]          # at most two streams at a time
    results, stats = srv.run(specs)
    assert stats["peak_hbm_bytes"] <= srv.budget
    assert stats["admission_waits"] > 0
    _check_exact(specs, results)


# ---- the native runtime (gdbg_server_*) ------------------------------------

@pytest.mark.parametrize("threads", [1, 3])
@pytest.mark.timeout(300)
def test_native_serving_matches_sequential_replay(cuda_ready, threads):
    specs = _specs(seed=9, n=10)
    srv = serving.NativeServer(G.BitStorage, G.CanLemireShifter, K=31, hbm_budget=8 << 30,
                               depth=3, dispatch_threads=threads)
    results, stats = srv.run(specs)
    assert stats["chunks"] == sum(len(s.chunks) for s in specs)
    assert stats["kmers"] == sum(s.n_kmers(31) for s in specs)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    _check_exact(specs, results)


def test_native_stream_alone_equals_stream_in_mix(cuda_ready):
    specs = _specs(seed=5)
    srv = serving.NativeServer(G.BitStorage, G.CanLemireShifter, K=31, hbm_budget=8 << 30,
                               dispatch_threads=2)
    mixed, _ = srv.run(specs)
    alone, _ = srv.run([specs[2]])
    for a, b in zip(alone[specs[2].sid], mixed[specs[2].sid]):
        assert np.array_equal(a.n_new, b.n_new)


def test_native_admission_by_hbm_budget(cuda_ready):
    specs = serving.make_streams(6, 7, reads_lo=1000, reads_hi=3000, chunk_lo=8, chunk_hi=256,
                                 table_lo_bits=16, table_hi_bits=20, mean_gap_s=0.002,
                                 genome_len=200_000, start_spread_s=0.001)
    srv = serving.NativeServer(G.BitStorage, G.CanLemireShifter, K=31, dispatch_threads=2)
    need = sorted(srv.footprints(specs))
    srv.budget = need[-1] + need[-2]          # at most two streams at a time
    results, stats = srv.run(specs)
    assert stats["peak_hbm_bytes"] <= srv.budget
    assert stats["admission_waits"] > 0 and stats["lazy_frees"] > 0
    _check_exact(specs, results)


def test_native_stream_over_budget_is_refused(cuda_ready):
    specs = _specs(seed=3, n=2)
    srv = serving.NativeServer(G.BitStorage, G.CanLemireShifter, K=31, hbm_budget=1 << 20)
    with pytest.raises(MemoryError):
        srv.run(specs)
