"""gdbg_insert_batch_noalloc: the insert entry point for callers that cannot
allocate device memory (a framework that owns every GPU byte through its own
pool, or a loop that must not pay cudaMalloc's device-wide synchronisation).

It is checked against the ordinary batch insert (gdbg_insert_batch) through
the C ABI: two batches in a row into caller-owned tables must give the same
per-read new-k-mer counts, the same n_unique / n_occupied increments and the
same table bytes, bit for bit.  The buffers handed to the entry point are
allocated by this test (through torch); the entry point itself allocates
nothing.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import goetia_gb300 as G
from goetia_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

u64p = _lib.u64p


def _layout(kind, sizes):
    offs = np.zeros(len(sizes) + 1, np.uint64)
    _lib.call("gdbg_noalloc_table_layout", kind, sizes.ctypes.data_as(u64p), len(sizes),
              offs.ctypes.data_as(u64p))
    return offs


@pytest.mark.parametrize("kind,storage", [(_lib.BYTE, G.ByteStorage), (_lib.BIT, G.BitStorage),
                                          (_lib.NIBBLE, G.NibbleStorage)])
def test_noalloc_matches_batch_insert(cuda_ready, kind, storage):
    import torch
    K = 31
    gen = synth.genome(150_000, 31)
    batches = [synth.rows_to_packed(synth.sample_reads(gen, 4000, 150, 0.01, 40 + i))
               for i in range(2)]
    sizes = np.asarray(storage.build(200_003, 4).get_tablesizes(), np.uint64)

    # the existing entry point
    ref = G.dBG[storage, G.CanLemireShifter].build(storage(tablesizes=sizes), K)
    ref_new, ref_stats = [], []
    for pr in batches:
        before = (ref.n_unique(), ref.n_occupied())
        ref_new.append(ref.insert_packed(pr))
        ref_stats.append((ref.n_unique() - before[0], ref.n_occupied() - before[1]))

    # the no-alloc entry point on caller-owned device buffers
    dev = torch.device("cuda", 0)
    offs = _layout(kind, sizes)
    tables = torch.zeros(int(offs[-1]), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    for pr, want_new, want_stats in zip(batches, ref_new, ref_stats):
        d_packed = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
        d_off = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
        d_new = torch.full((pr.n_reads,), -1, dtype=torch.int64, device=dev)
        d_stats = torch.full((3,), -1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize(dev)
        _lib.call("gdbg_insert_batch_noalloc", kind, _lib.CAN_LEMIRE, K,
                  sizes.ctypes.data_as(u64p), len(sizes), tables.data_ptr(), d_packed.data_ptr(),
                  d_packed.numel(), d_off.data_ptr(), pr.n_reads, d_new.data_ptr(),
                  d_stats.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        got_new = d_new.cpu().numpy().view(np.uint64)
        got_stats = d_stats.cpu().numpy().view(np.uint64)
        assert np.array_equal(got_new, want_new)
        assert (int(got_stats[0]), int(got_stats[1])) == want_stats
        assert int(got_stats[2]) == 0

    words = tables.cpu().numpy().view(np.uint8)
    for i, want in enumerate(ref.get_raw()):
        start = int(offs[i]) * 4
        assert np.array_equal(words[start:start + len(want)], want)


def test_noalloc_rejects_oversized_batches(cuda_ready):
    sizes = np.array([1009, 1013], np.uint64)
    n_reads = 131072 + 1
    offsets = np.zeros(n_reads + 1, np.uint64)
    with pytest.raises(G.GoetiaError) as e:
        _lib.call("gdbg_insert_batch_noalloc", _lib.BIT, _lib.CAN_LEMIRE, 31,
                  sizes.ctypes.data_as(u64p), 2, ctypes.c_void_p(1), ctypes.c_void_p(1), 1,
                  ctypes.c_void_p(1), n_reads, None, None, None)
    assert "maximum" in str(e.value)
    with pytest.raises(G.GoetiaError):
        _lib.call("gdbg_insert_batch_noalloc", _lib.BIT, _lib.CAN_LEMIRE, 31,
                  sizes.ctypes.data_as(u64p), 9, ctypes.c_void_p(1), ctypes.c_void_p(1), 1,
                  ctypes.c_void_p(1), 1, None, None, None)
