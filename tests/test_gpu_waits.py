"""Bounded device waits driven to their limits, with no GPU fault.

Every spin-wait in the insert kernels has a poll limit: the persistent
insert's grid barrier and the bucketed insert's waits on its shared-memory
bulk copies.  gdbg_set_wait_limits lowers a limit to a few polls; the wait
then runs out on an ordinary batch.  The kernel must record the timeout bit
in the handle's status word and return, the next synchronising call must
raise GDBG_ERR_DEVICE carrying that bit, and the same handle must stay
usable: after gdbg_reset (and the default limits back) the next batch gives
exactly the oracle's per-read new counts, tables and counters.  A timed-out
persistent run leaves its claims map behind; the kernel marks it stale, so
the following run starts from a cleared map.
"""
import re

import numpy as np
import pytest

import oracle
import goetia_gb300 as G
from goetia_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

BARRIER_TIMEOUT = 4
COPY_TIMEOUT = 16


def _status_bits(err):
    m = re.search(r"device status 0x([0-9a-f]+)", str(err))
    assert m, str(err)
    return int(m.group(1), 16)


def _device_batch(pr, dev):
    import torch
    d_packed = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
    d_off = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
    d_new = torch.zeros(max(pr.n_reads, 1), dtype=torch.int64, device=dev)
    return d_packed, d_off, d_new


def _insert_device(g, pr, dev):
    d_packed, d_off, d_new = _device_batch(pr, dev)
    g.insert_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), pr.n_reads,
                    n_new_ptr=d_new.data_ptr())
    return d_packed, d_off, d_new


def _expect_oracle(g, kind, sizes, pr, K, canonical):
    ref = oracle.Storage(kind, sizes)
    _, want = ref.insert_reads(canonical, K, pr.packed, pr.offsets)
    before = (g.n_unique(), g.n_occupied())
    got = g.insert_packed(pr)
    assert np.array_equal(got, want)
    for a, b in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, b)
    n_u, n_o = ref.stats()
    assert (g.n_unique() - before[0], g.n_occupied() - before[1]) == (n_u, n_o)


def test_grid_barrier_limit_runs_out_then_handle_recovers(cuda_ready):
    import torch
    dev = torch.device("cuda", 0)
    gen = synth.genome(400_000, 71)
    a = synth.rows_to_packed(synth.sample_reads(gen, 6000, 150, 0.01, 72))
    b = synth.rows_to_packed(synth.sample_reads(gen, 6000, 150, 0.01, 73))
    sizes = oracle.primes(4, 1 << 21)
    g = G.dBG[G.ByteStorage, G.CanLemireShifter].build(G.ByteStorage(tablesizes=sizes), 31)
    g.set_insert_path("persistent")
    g.set_insert_schedule(65536, 4)   # 11 windows, three barrier waits each
    g.set_wait_limits(barrier_polls=1)
    bufs = _insert_device(g, a, dev)
    with pytest.raises(G.GoetiaError) as e:
        g.synchronize()
    assert e.value.code == _lib.ERR_DEVICE
    assert _status_bits(e.value) & BARRIER_TIMEOUT
    del bufs
    # the status was read and cleared: the handle answers again
    g.synchronize()
    g.set_wait_limits(0, 0)
    g.reset()
    # the aborted run's claims must not leak into this one (same path)
    _expect_oracle(g, "byte", sizes, b, 31, True)


def test_bulk_copy_limit_runs_out_then_handle_recovers(cuda_ready):
    import torch
    dev = torch.device("cuda", 0)
    gen = synth.genome(2_000_000, 81)
    a = synth.rows_to_packed(synth.sample_reads(gen, 40_000, 150, 0.01, 82))
    b = synth.rows_to_packed(synth.sample_reads(gen, 40_000, 150, 0.01, 83))
    sizes = oracle.primes(4, 1 << 22)
    g = G.dBG[G.ByteStorage, G.CanLemireShifter].build(G.ByteStorage(tablesizes=sizes), 31)
    g.set_insert_path("bucketed")
    g.set_wait_limits(copy_polls=1)
    bufs = _insert_device(g, a, dev)
    with pytest.raises(G.GoetiaError) as e:
        g.synchronize()
    assert e.value.code == _lib.ERR_DEVICE
    assert _status_bits(e.value) & COPY_TIMEOUT
    del bufs
    g.synchronize()
    g.set_wait_limits(0, 0)
    g.reset()
    _expect_oracle(g, "byte", sizes, b, 31, True)
    # and the same handle's segmented path is exact on a second batch
    g2 = g.clone()
    g2.set_insert_path("bucketed")
    _expect_oracle(g2, "byte", sizes, a, 31, True)


def test_default_limits_do_not_fire(cuda_ready):
    """The same batches with the default limits: no status bit, exact."""
    gen = synth.genome(400_000, 71)
    a = synth.rows_to_packed(synth.sample_reads(gen, 6000, 150, 0.01, 72))
    sizes = oracle.primes(4, 1 << 21)
    for path in ("persistent", "bucketed"):
        g = G.dBG[G.ByteStorage, G.CanLemireShifter].build(G.ByteStorage(tablesizes=sizes), 31)
        g.set_insert_path(path)
        g.set_insert_schedule(65536, 4)
        _expect_oracle(g, "byte", sizes, a, 31, True)
        assert g.device_status() == 0
