"""Serving loop: many concurrent sample streams, each with its own dBG resident
in HBM, fed with read chunks as they arrive.

The reference's streaming driver (goetia/processors.py:39-498,
AsyncSequenceProcessor) consumes one sample at a time in a worker thread and
reports progress per interval of k-mers.  Here one process serves many
samples at once on one GPU:

* admission: a stream is admitted when its tables and scratch fit in the HBM
  budget; otherwise it waits until a finished stream releases its memory;
* continuous batching: every admitted stream has its own CUDA stream; a chunk
  is dispatched as soon as it arrives (host pinned staging, then one
  asynchronous library call that queues the H2D copy, the insert and the D2H
  copy of the per-read new-k-mer counts, then an event), up to `depth` chunks
  of a stream in flight, so chunks of different streams overlap on the device
  while each stream's chunks apply in arrival order;
* admission ahead of arrival: while no arrived chunk waits, streams whose
  first chunk is due within `lookahead_s` are admitted early, so building a
  stream's graph does not hold up other streams' chunks;
* completion: events are polled; a chunk's latency is completion time minus
  arrival time;
* release: a finished stream's budget share is returned at once, but its
  device memory is freed lazily -- only when an admission needs the room, or
  at the end of the run -- because freeing device memory waits for every
  stream's in-flight work and would stall the dispatch of all other streams.

Per-chunk new counts equal a sequential replay of each stream, whatever the
mix (tests/test_gpu_serving.py).
"""
import collections
import dataclasses
import time

import numpy as np

from . import dbg as D
from .reads import PackedReads


@dataclasses.dataclass
class StreamSpec:
    """One sample: its table size and its chunks with arrival times (seconds
    from the start of the run)."""
    sid: int
    max_table: int
    chunks: list            # list of PackedReads
    arrivals: list          # seconds, non-decreasing

    def n_kmers(self, K):
        return sum(c.n_kmers(K) for c in self.chunks)


@dataclasses.dataclass
class ChunkResult:
    sid: int
    index: int
    n_reads: int
    n_kmers: int
    n_new: np.ndarray
    arrival: float
    done: float

    @property
    def latency(self):
        return self.done - self.arrival


class _Slot:
    """Pinned host staging of one in-flight chunk (packed words, offsets, new
    counts); the device side lives in the graph's staging buffers."""

    def __init__(self, torch, max_words, max_reads):
        self.h_packed = torch.empty(max_words, dtype=torch.int32).pin_memory()
        self.h_off = torch.empty(max_reads + 1, dtype=torch.int64).pin_memory()
        self.h_new = torch.empty(max_reads, dtype=torch.int64).pin_memory()
        self.packed = self.h_packed.numpy()
        self.off = self.h_off.numpy()
        self.new = self.h_new.numpy()
        self.event = torch.cuda.Event()   # recorded after the slot's chunk


class _Stream:
    def __init__(self, spec, server):
        torch = server.torch
        self.spec = spec
        storage = server.storage_type.build(spec.max_table, server.n_tables)
        self.graph = D.dBG[server.storage_type, server.shifter_type].build(storage, server.K)
        self.graph.set_insert_path("windowed")
        self.graph.set_insert_schedule(server.window, 4)
        self.cuda = torch.cuda.Stream(server.dev)
        self.graph.set_stream(self.cuda.cuda_stream)
        max_reads = max(c.n_reads for c in spec.chunks)
        max_words = max(c.packed.size for c in spec.chunks)
        self.slots = [_Slot(torch, max_words, max_reads) for _ in range(server.depth)]
        self.free = collections.deque(range(server.depth))
        self.inflight = collections.deque()      # (event, slot, index)
        self.next_chunk = 0                      # next chunk to dispatch
        self.done_chunks = 0
        self.results = []
        # grow the graph's scratch to the largest chunk now, so no device
        # allocation (and its device-wide synchronisation) happens while
        # serving
        self.graph.reserve(max_reads, max(c.n_kmers(server.K) for c in spec.chunks))
        self.graph.reserve_staging(max_words, max_reads)

    def table_bytes(self):
        return sum(self.graph.table_bytes())


def stream_footprint(storage_type, max_table, n_tables, window, n_tables_scratch=None):
    """HBM bytes a stream holds: tables plus the windowed insert's scratch."""
    sizes = storage_type.build(max_table, n_tables).get_tablesizes()
    per = {D.BitStorage: lambda p: p // 8 + 1, D.ByteStorage: lambda p: p,
           D.NibbleStorage: lambda p: p // 2 + 1}[storage_type]
    tables = sum((per(p) + 255) // 256 * 256 for p in sizes)
    slots = 1
    while slots < 2 * window * n_tables:
        slots *= 2
    scratch = slots * 8 * 5 // 4 + window * 4 * (1 + n_tables)
    return tables + scratch


class Server:
    """Continuous-batching server for many dBG streams on one GPU."""

    def __init__(self, storage_type=D.BitStorage, shifter_type=D.CanLemireShifter, K=31,
                 n_tables=4, hbm_budget=16 << 30, depth=2, window=262144, device=0,
                 lookahead_s=0.05):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.storage_type = storage_type
        self.shifter_type = shifter_type
        self.K = K
        self.n_tables = n_tables
        self.budget = hbm_budget
        self.depth = depth
        self.window = window
        self.lookahead = lookahead_s

    def footprint(self, spec):
        """Device bytes of a stream: tables and insert scratch, plus the
        staging of its largest chunk."""
        return stream_footprint(self.storage_type, spec.max_table, self.n_tables, self.window) + \
            (max(c.packed.size for c in spec.chunks) * 4 +
             (2 * max(c.n_reads for c in spec.chunks) + 1) * 8)

    def run(self, specs, time_scale=1.0, max_seconds=600.0):
        """Serve every stream's chunks at their arrival times.  Returns
        (results, stats): results per stream id (list of ChunkResult in chunk
        order), stats with latency percentiles, throughput and admission.
        Python's cyclic garbage collector is paused for the run (a full
        collection would stall dispatch for tens of milliseconds)."""
        import gc
        was_enabled = gc.isenabled()
        gc.disable()
        try:
            return self._run(specs, time_scale, max_seconds)
        finally:
            if was_enabled:
                gc.enable()

    def _run(self, specs, time_scale, max_seconds):
        torch = self.torch
        order = sorted(specs, key=lambda s: s.arrivals[0])
        waiting = collections.deque(order)       # not yet admitted
        active = {}
        zombies = []                             # finished, memory not yet freed
        zombie_bytes = 0
        used = 0
        peak_used = 0
        results = {}
        admitted_at = {}
        waited = set()
        freed_at = []
        admit_s, dispatch_s, delay = [], [], []    # host-side timings
        total_kmers = 0
        lat = []
        t0 = time.perf_counter()
        first_dispatch = None
        last_done = None
        while waiting or active:
            now = (time.perf_counter() - t0) / time_scale
            if now > max_seconds:
                raise TimeoutError("serving run exceeded its time limit")
            # admission: streams whose first chunk has arrived, in arrival
            # order; ahead of their arrival when nothing is waiting to go
            idle = all(not (st.free and st.next_chunk < len(st.spec.chunks)
                            and st.spec.arrivals[st.next_chunk] <= now)
                       for st in active.values())
            horizon = now + (self.lookahead if idle else 0.0)
            while waiting and waiting[0].arrivals[0] <= horizon:
                spec = waiting[0]
                need = self.footprint(spec)
                if need > self.budget:
                    raise MemoryError(f"stream {spec.sid} needs {need} bytes, over the budget")
                if used + need > self.budget:
                    if spec.arrivals[0] <= now:
                        waited.add(spec.sid)
                    break
                if zombies and used + zombie_bytes + need > self.budget:
                    zombies.clear()                 # frees their device memory
                    zombie_bytes = 0
                    freed_at.append(now)
                waiting.popleft()
                ta = time.perf_counter()
                st = _Stream(spec, self)
                admit_s.append(time.perf_counter() - ta)
                st.need = need
                used += need
                peak_used = max(peak_used, used + zombie_bytes)   # held on the device
                active[spec.sid] = st
                admitted_at[spec.sid] = now
            # dispatch arrived chunks
            for st in active.values():
                spec = st.spec
                while (st.free and st.next_chunk < len(spec.chunks)
                       and spec.arrivals[st.next_chunk] <= now):
                    i = st.next_chunk
                    c = spec.chunks[i]
                    td = time.perf_counter()
                    delay.append((td - t0) / time_scale - spec.arrivals[i])
                    si = st.free.popleft()
                    slot = st.slots[si]
                    nw, nr = c.packed.size, c.n_reads
                    slot.packed[:nw] = c.packed.view(np.int32)
                    slot.off[:nr + 1] = c.offsets.view(np.int64)
                    st.graph.insert_async(slot.h_packed.data_ptr(), nw, slot.h_off.data_ptr(), nr,
                                          c.n_kmers(self.K), slot.h_new.data_ptr(),
                                          stream=st.cuda.cuda_stream)
                    slot.event.record(st.cuda)
                    st.inflight.append((slot.event, si, i))
                    st.next_chunk += 1
                    dispatch_s.append(time.perf_counter() - td)
                    if first_dispatch is None:
                        first_dispatch = time.perf_counter()
            # completions (in order per stream)
            finished = []
            for sid, st in active.items():
                while st.inflight and st.inflight[0][0].query():
                    ev, si, i = st.inflight.popleft()
                    done = (time.perf_counter() - t0) / time_scale
                    c = st.spec.chunks[i]
                    slot = st.slots[si]
                    r = ChunkResult(sid, i, c.n_reads, c.n_kmers(self.K),
                                    slot.new[:c.n_reads].view(np.uint64).copy(),
                                    st.spec.arrivals[i], done)
                    st.results.append(r)
                    lat.append(r.latency)
                    total_kmers += r.n_kmers
                    st.free.append(si)
                    last_done = time.perf_counter()
                if st.next_chunk == len(st.spec.chunks) and not st.inflight:
                    finished.append(sid)
            for sid in finished:
                st = active.pop(sid)
                results[sid] = st.results
                used -= st.need
                zombies.append(st)
                zombie_bytes += st.need
                del st
        lat_ms = np.array(lat) * 1000.0 * time_scale
        span = (last_done - first_dispatch) if first_dispatch and last_done else 0.0
        zombies.clear()
        stats = {
            "chunks": len(lat),
            "kmers": total_kmers,
            "kmers_per_s": total_kmers / span if span > 0 else 0.0,
            "p50_ms": float(np.percentile(lat_ms, 50)) if len(lat_ms) else 0.0,
            "p99_ms": float(np.percentile(lat_ms, 99)) if len(lat_ms) else 0.0,
            "max_ms": float(lat_ms.max()) if len(lat_ms) else 0.0,
            "peak_hbm_bytes": peak_used,
            "admission_waits": len(waited),
            "lazy_frees": len(freed_at),
            "wall_s": span,
            # host side: stream admission (graph creation), per-chunk dispatch
            # work, and the wait from a chunk's arrival to its dispatch
            "admit_ms_max": 1e3 * max(admit_s) if admit_s else 0.0,
            "admit_ms_total": 1e3 * sum(admit_s),
            "dispatch_ms_p99": float(np.percentile(dispatch_s, 99)) * 1e3 if dispatch_s else 0.0,
            "dispatch_delay_ms_p99": (float(np.percentile(delay, 99)) * 1e3 * time_scale
                                      if delay else 0.0),
        }
        return results, stats


class NativeServer:
    """The same serving loop run by the library's native runtime
    (gdbg_server_*): admission, dispatch and completion polling in C++
    threads, so the per-chunk host cost is a copy into pinned staging and one
    asynchronous insert call instead of a Python iteration.  Same run(specs)
    contract as Server: chunks are released at their arrival times and each
    result equals a sequential replay of its stream."""

    def __init__(self, storage_type=D.BitStorage, shifter_type=D.CanLemireShifter, K=31,
                 n_tables=4, hbm_budget=16 << 30, depth=4, dispatch_threads=2, device=0):
        import torch
        self.torch = torch
        self.device = device
        self.kinds = (storage_type.kind, shifter_type.kind)
        self.K = K
        self.n_tables = n_tables
        self.budget = hbm_budget
        self.depth = depth
        self.dispatch_threads = dispatch_threads

    def footprints(self, specs):
        """The native runtime's HBM budget share of each stream (bytes)."""
        import ctypes
        from . import _lib
        h = ctypes.c_void_p()
        _lib.call("gdbg_server_create", self.kinds[0], self.kinds[1], self.K, self.n_tables,
                  (1 << 63), self.depth, 1, ctypes.byref(h))
        try:
            out = []
            for spec in specs:
                _lib.call("gdbg_server_stream", h, spec.sid, spec.max_table,
                          max(c.n_reads for c in spec.chunks),
                          max(c.packed.size for c in spec.chunks))
                b = ctypes.c_uint64()
                _lib.call("gdbg_server_stream_bytes", h, spec.sid, ctypes.byref(b))
                out.append(int(b.value))
            return out
        finally:
            _lib.call("gdbg_server_destroy", h)

    def run(self, specs, max_seconds=600.0):
        import ctypes
        from . import _lib
        self.torch.cuda.set_device(self.device)
        h = ctypes.c_void_p()
        _lib.call("gdbg_server_create", self.kinds[0], self.kinds[1], self.K, self.n_tables,
                  int(self.budget), self.depth, self.dispatch_threads, ctypes.byref(h))
        try:
            outs, index = {}, []
            for spec in specs:
                _lib.call("gdbg_server_stream", h, spec.sid, spec.max_table,
                          max(c.n_reads for c in spec.chunks),
                          max(c.packed.size for c in spec.chunks))
            for spec in specs:
                outs[spec.sid] = []
                for i, (c, t) in enumerate(zip(spec.chunks, spec.arrivals)):
                    nn = np.zeros(max(c.n_reads, 1), np.uint64)
                    outs[spec.sid].append(nn)
                    tag = len(index)
                    index.append((spec.sid, i, c.n_reads, c.n_kmers(self.K), float(t)))
                    _lib.call("gdbg_server_submit", h, spec.sid, c.packed.ctypes.data,
                              c.packed.size, c.offsets.ctypes.data, c.n_reads, index[-1][3],
                              float(t), nn.ctypes.data, tag)
                _lib.call("gdbg_server_finish", h, spec.sid)
            _lib.call("gdbg_server_start", h)
            _lib.call("gdbg_server_wait", h, float(max_seconds))
            n = len(index)
            tags = np.zeros(max(n, 1), np.uint64)
            lat = np.zeros(max(n, 1), np.float64)
            done = np.zeros(max(n, 1), np.float64)
            ok = np.zeros(max(n, 1), np.int32)
            got = ctypes.c_uint64()
            _lib.call("gdbg_server_poll", h, tags.ctypes.data, lat.ctypes.data, done.ctypes.data,
                      ok.ctypes.data, n, ctypes.byref(got))
            rep = _lib.ServerReport()
            _lib.call("gdbg_server_stats", h, ctypes.byref(rep))
            err = _lib.load().gdbg_server_last_error(h).decode(errors="replace")
        finally:
            _lib.call("gdbg_server_destroy", h)
        m = int(got.value)
        if m != n or not ok[:m].all() or rep.chunks_failed or rep.device_status:
            raise _lib.GoetiaError(_lib.ERR_DEVICE,
                                   f"serving: {m} of {n} chunks completed, {rep.chunks_failed} "
                                   f"failed, device status {rep.device_status:#x}: {err}")
        results = {spec.sid: [None] * len(spec.chunks) for spec in specs}
        for k in range(m):
            sid, i, nr, nk, t = index[int(tags[k])]
            results[sid][i] = ChunkResult(sid, i, nr, nk, outs[sid][i][:nr], t, t + float(lat[k]))
        lat_ms = lat[:m] * 1e3
        span = rep.last_done_s - rep.first_dispatch_s
        stats = {
            "chunks": m, "kmers": int(rep.kmers_done),
            "kmers_per_s": rep.kmers_done / span if span > 0 else 0.0,
            "p50_ms": float(np.percentile(lat_ms, 50)) if m else 0.0,
            "p99_ms": float(np.percentile(lat_ms, 99)) if m else 0.0,
            "max_ms": float(lat_ms.max()) if m else 0.0,
            "peak_hbm_bytes": int(rep.peak_hbm_bytes),
            "admission_waits": int(rep.admission_waits), "lazy_frees": int(rep.lazy_frees),
            "wall_s": span,
            "admit_ms_max": 1e3 * rep.admit_s_max, "admit_ms_total": 1e3 * rep.admit_s_total,
            "dispatch_ms_mean": 1e3 * rep.dispatch_s_total / max(m, 1),
            "dispatch_ms_max": 1e3 * rep.dispatch_s_max,
            "dispatch_threads": self.dispatch_threads,
        }
        return results, stats


def replay(spec, storage_type=D.BitStorage, shifter_type=D.CanLemireShifter, K=31, n_tables=4):
    """Sequential replay of one stream: its chunks inserted one after another
    into a fresh graph (the reference's order).  Returns per-chunk n_new."""
    storage = storage_type.build(spec.max_table, n_tables)
    g = D.dBG[storage_type, shifter_type].build(storage, K)
    g.set_insert_path("windowed")
    return [g.insert_packed(c) for c in spec.chunks]


def make_streams(n_streams, seed, reads_lo, reads_hi, chunk_lo, chunk_hi, table_lo_bits,
                 table_hi_bits, mean_gap_s, genome_len=2_000_000, read_len=150, sub_rate=0.01,
                 start_spread_s=1.0, max_arrival_s=None, threads=None, reads_cache=None):
    """Seeded serving workload: stream sizes log-uniform in [reads_lo, reads_hi],
    chunk sizes log-uniform in [chunk_lo, chunk_hi], table sizes log-uniform
    in [2^table_lo_bits, 2^table_hi_bits] per table, Poisson chunk arrivals
    with mean gap mean_gap_s, stream starts uniform over start_spread_s.
    Each stream samples its reads (either strand, i.i.d. substitutions) from
    its own random genome with the multi-threaded generator; a chunk is a
    view of the stream's packed reads.  max_arrival_s keeps only the chunks
    that arrive before it (a time window of the same streams).  reads_cache
    (a dict) keeps each stream's generated reads for later calls with the
    same seed and sizes."""
    from . import synth
    rng = np.random.default_rng(seed)
    specs = []
    for s in range(n_streams):
        g = synth.genome(genome_len, seed * 1000 + s)
        n_reads = int(np.exp(rng.uniform(np.log(reads_lo), np.log(reads_hi))))
        bits = rng.uniform(table_lo_bits, table_hi_bits)
        max_table = int(2 ** bits)
        key = (seed, s, n_reads, read_len, sub_rate, genome_len)
        reads = reads_cache.get(key) if reads_cache is not None else None
        if reads is None:
            reads = synth.sample_reads_packed(g, n_reads, read_len, sub_rate, seed * 7919 + s,
                                              threads=threads)
            if reads_cache is not None:
                reads_cache[key] = reads
        chunks, arrivals = [], []
        t = rng.uniform(0.0, start_spread_s)
        pos = 0
        while pos < n_reads:
            n = int(np.exp(rng.uniform(np.log(chunk_lo), np.log(chunk_hi))))
            n = max(1, min(n, n_reads - pos))
            if max_arrival_s is not None and t >= max_arrival_s:
                break
            chunks.append(reads.slice(pos, pos + n))
            arrivals.append(t)
            t += rng.exponential(mean_gap_s)
            pos += n
        if chunks:
            specs.append(StreamSpec(s, max_table, chunks, arrivals))
    return specs
