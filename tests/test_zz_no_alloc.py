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


def _noalloc(kind, shifter, K, sizes, tables, pr, dev, stream, with_new=True, with_stats=True):
    """One call of the entry point on device copies of a batch; returns the
    per-read new counts and the stats words (None where not asked for)."""
    import torch
    d_packed = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
    d_off = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
    d_new = torch.full((max(pr.n_reads, 1),), -1, dtype=torch.int64, device=dev)
    d_stats = torch.full((3,), -1, dtype=torch.int64, device=dev)
    torch.cuda.synchronize(dev)
    _lib.call("gdbg_insert_batch_noalloc", kind, shifter, K, sizes.ctypes.data_as(u64p),
              len(sizes), tables.data_ptr(), d_packed.data_ptr(), d_packed.numel(),
              d_off.data_ptr(), pr.n_reads, d_new.data_ptr() if with_new else None,
              d_stats.data_ptr() if with_stats else None, stream.cuda_stream)
    stream.synchronize()
    got_new = d_new.cpu().numpy().view(np.uint64)[:pr.n_reads] if with_new else None
    got_stats = d_stats.cpu().numpy().view(np.uint64) if with_stats else None
    return got_new, got_stats


SHAPES = [
    # kind, storage, shifter, K, table sizes near, n_tables
    (_lib.BYTE, G.ByteStorage, G.CanLemireShifter, 31, 200_003, 4),
    (_lib.BIT, G.BitStorage, G.CanLemireShifter, 31, 200_003, 4),
    (_lib.NIBBLE, G.NibbleStorage, G.CanLemireShifter, 31, 200_003, 4),
    (_lib.NIBBLE, G.NibbleStorage, G.FwdLemireShifter, 21, 300_007, 3),
    (_lib.BIT, G.BitStorage, G.CanLemireShifter, 64, 400_009, 8),
    (_lib.BYTE, G.ByteStorage, G.FwdLemireShifter, 64, 150_001, 4),
]


@pytest.mark.parametrize("kind,storage,shifter,K,near,n_tables", SHAPES)
def test_noalloc_matches_batch_insert(cuda_ready, kind, storage, shifter, K, near, n_tables):
    """Two batches in a row (each about 480k k-mers, eight 65,536-k-mer
    windows) against gdbg_insert_batch on the same reads."""
    import torch
    gen = synth.genome(150_000, 31)
    batches = [synth.rows_to_packed(synth.sample_reads(gen, 4000, 150, 0.01, 40 + i))
               for i in range(2)]
    sizes = np.asarray(storage.build(near, n_tables).get_tablesizes(), np.uint64)
    code = _lib.CAN_LEMIRE if shifter is G.CanLemireShifter else _lib.FWD_LEMIRE

    # the existing entry point
    ref = G.dBG[storage, shifter].build(storage(tablesizes=sizes), K)
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
        got_new, got_stats = _noalloc(kind, code, K, sizes, tables, pr, dev, stream)
        assert np.array_equal(got_new, want_new)
        assert (int(got_stats[0]), int(got_stats[1])) == want_stats
        assert int(got_stats[2]) == 0

    words = tables.cpu().numpy().view(np.uint8)
    for i, want in enumerate(ref.get_raw()):
        start = int(offs[i]) * 4
        assert np.array_equal(words[start:start + len(want)], want)


def test_noalloc_without_outputs_and_across_the_epoch_wrap(cuda_ready):
    """n_new and stats NULL, three batches of about 6M k-mers each: 276
    windows in all, so the claims map's epochs wrap past 127 between calls.
    The tables must equal gdbg_insert_batch's after the same batches."""
    import torch
    gen = synth.genome(2_000_000, 33)
    batches = [synth.rows_to_packed(synth.sample_reads(gen, 50_000, 150, 0.01, 50 + i))
               for i in range(3)]
    sizes = np.asarray(G.ByteStorage.build(1 << 22, 4).get_tablesizes(), np.uint64)
    ref = G.dBG[G.ByteStorage, G.CanLemireShifter].build(G.ByteStorage(tablesizes=sizes), 31)
    for pr in batches:
        ref.insert_packed(pr)
    dev = torch.device("cuda", 0)
    offs = _layout(_lib.BYTE, sizes)
    tables = torch.zeros(int(offs[-1]), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    for pr in batches:
        _noalloc(_lib.BYTE, _lib.CAN_LEMIRE, 31, sizes, tables, pr, dev, stream,
                 with_new=False, with_stats=False)
    # one more call with outputs: its new counts follow on from the same state
    extra = synth.rows_to_packed(synth.sample_reads(gen, 4000, 150, 0.01, 59))
    want_new = ref.insert_packed(extra)
    got_new, got_stats = _noalloc(_lib.BYTE, _lib.CAN_LEMIRE, 31, sizes, tables, extra, dev, stream)
    assert np.array_equal(got_new, want_new)
    assert int(got_stats[2]) == 0
    words = tables.cpu().numpy().view(np.uint8)
    for i, want in enumerate(ref.get_raw()):
        start = int(offs[i]) * 4
        assert np.array_equal(words[start:start + len(want)], want)


def test_noalloc_bad_offsets_are_reported(cuda_ready):
    """A read whose end runs past the packed stream: like
    gdbg_insert_batch_device, the read counts as zero k-mers, the others are
    inserted, and status bit 8 reports it -- in stats[2], or, with stats
    NULL, as GDBG_ERR_DEVICE from the call itself."""
    import torch
    gen = synth.genome(150_000, 35)
    pr = synth.rows_to_packed(synth.sample_reads(gen, 2000, 150, 0.01, 36))
    bad = G.PackedReads(pr.packed, pr.offsets.copy())
    bad.offsets[1000] = np.uint64(len(pr.packed) * 16 + 1000)   # read 999 ends past the stream
    sizes = np.asarray(G.BitStorage.build(100_003, 4).get_tablesizes(), np.uint64)
    dev = torch.device("cuda", 0)

    # the existing device entry point on the same batch
    ref = G.dBG[G.BitStorage, G.CanLemireShifter].build(G.BitStorage(tablesizes=sizes), 31)
    d_packed = torch.from_numpy(bad.packed.view(np.int32)).to(dev)
    d_off = torch.from_numpy(bad.offsets.view(np.int64)).to(dev)
    d_new = torch.zeros(bad.n_reads, dtype=torch.int64, device=dev)
    ref.insert_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), bad.n_reads,
                      n_new_ptr=d_new.data_ptr())
    with pytest.raises(G.GoetiaError) as e:
        ref.synchronize()
    assert e.value.code == _lib.ERR_DEVICE
    want_new = d_new.cpu().numpy().view(np.uint64)

    offs = _layout(_lib.BIT, sizes)
    tables = torch.zeros(int(offs[-1]), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    got_new, got_stats = _noalloc(_lib.BIT, _lib.CAN_LEMIRE, 31, sizes, tables, bad, dev, stream)
    assert int(got_stats[2]) & 8
    assert np.array_equal(got_new, want_new)
    words = tables.cpu().numpy().view(np.uint8)
    for i, want in enumerate(ref.get_raw()):
        start = int(offs[i]) * 4
        assert np.array_equal(words[start:start + len(want)], want)
    # without a stats buffer the call itself reports the failed check
    with pytest.raises(G.GoetiaError) as e:
        _noalloc(_lib.BIT, _lib.CAN_LEMIRE, 31, sizes, tables, bad, dev, stream,
                 with_stats=False)
    assert e.value.code == _lib.ERR_DEVICE
    # and the next good call on the shared scratch is clean again
    _, st = _noalloc(_lib.BIT, _lib.CAN_LEMIRE, 31, sizes, tables, pr, dev, stream)
    assert int(st[2]) == 0


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
