"""Batched insert of read streams with uneven lengths: fixed-capacity batches
replayed through a captured CUDA graph, with an autotuner for the schedule.

The reference inserts one read per call (InserterProcessor::process_sequence,
include/goetia/processors.hh:304-331).  Here reads are grouped into batches
of at most `max_reads` reads and `max_bases` bases; every batch is copied into
the same device buffers (short batches are padded with empty reads) and the
whole insert -- k-mer prefix, partition or probe/commit passes, apply -- is
replayed as one CUDA graph.  The kernels bound their work by the batch's
device-side k-mer count, so one capture serves every batch that fits the
capacity.  Per-read new-k-mer counts come back in batch order, identical to
inserting the reads one by one.
"""
import json
import os
import time

import numpy as np

from . import _lib
from .reads import PackedReads


def split_batches(reads, max_reads, max_bases):
    """Cut a PackedReads into consecutive batches within the capacity (a read
    longer than max_bases is rejected)."""
    off = reads.offsets.astype(np.int64)
    lens = np.diff(off)
    if len(lens) and lens.max() > max_bases:
        raise ValueError("a read is longer than the batch base capacity")
    out, r = [], 0
    n = len(lens)
    while r < n:
        e = min(n, r + max_reads)
        # largest e with off[e] - off[r] <= max_bases
        lim = off[r] + max_bases
        e = min(e, int(np.searchsorted(off, lim, side="right")) - 1)
        e = max(e, r + 1)
        b0, b1 = int(off[r]), int(off[e])
        w0 = b0 // 16
        words = reads.packed[w0:(b1 + 15) // 16 + 1]
        sub_off = (off[r:e + 1] - 16 * w0).astype(np.uint64)
        out.append((r, PackedReads(np.ascontiguousarray(words, np.uint32), sub_off)))
        r = e
    return out


def bucketed_fits(graph, max_kmers, bucket_bits=0):
    """Whether the bucketed path takes batches of up to max_kmers k-mers on
    this graph (at most 8 tables, global cell ids and record indices below
    2^32)."""
    from . import dbg as D
    st = type(graph).storage_type
    fs = bucket_bits or {D.BitStorage: 19, D.ByteStorage: 16, D.NibbleStorage: 17}[st]
    sizes = graph.storage.tablesizes
    if len(sizes) > 8 or max_kmers * len(sizes) >= 1 << 32:
        return False
    return sum(((p + (1 << fs) - 1) >> fs) << fs for p in sizes) <= 1 << 32


class BatchedInserter:
    """Fixed-capacity batch insert into one graph, optionally as a CUDA graph.

    graph      a goetia_gb300 dBG
    max_reads  reads per batch (short batches are padded with empty reads)
    max_bases  bases per batch
    use_graph  capture the insert once and replay it per batch.  Replay needs
               an insert path that keeps no per-batch state on the host: the
               persistent fused kernel (one cooperative launch per batch,
               its claims epoch kept on the device) or a bucketed path; any
               other path is switched to the bucketed one (and replay is
               turned off when the tables do not fit it).
    """

    def __init__(self, graph, max_reads, max_bases, use_graph=True, device=0):
        import torch
        self.torch = torch
        self.g = graph
        self.K = graph.K
        self.max_reads = int(max_reads)
        self.max_bases = int(max_bases)
        self.max_words = self.max_bases // 16 + 4
        self.max_kmers = max(self.max_bases - self.K + 1, 1)
        dev = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(dev)
        graph.set_stream(self.stream.cuda_stream)
        self.d_packed = torch.zeros(self.max_words, dtype=torch.int32, device=dev)
        self.d_off = torch.zeros(self.max_reads + 1, dtype=torch.int64, device=dev)
        self.d_new = torch.zeros(self.max_reads, dtype=torch.int64, device=dev)
        # two pinned staging sets: insert_stream fills one on the host while
        # the batch staged from the other is on the GPU
        self.h_packed = [torch.zeros(self.max_words, dtype=torch.int32).pin_memory() for _ in range(2)]
        self.h_off = [torch.zeros(self.max_reads + 1, dtype=torch.int64).pin_memory() for _ in range(2)]
        self.h_new = [torch.zeros(self.max_reads, dtype=torch.int64).pin_memory() for _ in range(2)]
        self.done = [torch.cuda.Event(), torch.cuda.Event()]
        self.use_graph = use_graph
        if use_graph and str(graph.insert_path()) != "persistent":
            if bucketed_fits(graph, self.max_kmers, getattr(graph, "_bucket_bits", 0)):
                if not str(graph.insert_path()).startswith("bucketed"):
                    graph.set_insert_path("bucketed")
            else:
                self.use_graph = False
        self.cuda_graph = None
        self.launches = 0

    def _launch(self):
        self.g.insert_device(self.d_packed.data_ptr(), self.max_words, self.d_off.data_ptr(),
                             self.max_reads, n_kmers=self.max_kmers,
                             n_new_ptr=self.d_new.data_ptr(), stream=self.stream.cuda_stream)

    def _fill(self, batch, s):
        """Host side: the batch into pinned staging set s."""
        nw, nr = batch.packed.size, batch.n_reads
        if nr > self.max_reads or batch.n_bases > self.max_bases:
            raise ValueError("batch exceeds the inserter's capacity")
        self.h_packed[s][:nw].numpy()[:] = batch.packed.view(np.int32)
        off = self.h_off[s].numpy()
        off[:nr + 1] = batch.offsets.view(np.int64)
        off[nr + 1:] = off[nr]          # padding: empty reads

    def _submit(self, batch, s):
        """Stream side: copy staging set s in, insert, copy the new counts out
        into set s; done[s] marks the end."""
        torch = self.torch
        nw, nr = batch.packed.size, batch.n_reads
        with torch.cuda.stream(self.stream):
            self.d_packed[:nw].copy_(self.h_packed[s][:nw], non_blocking=True)
            self.d_off.copy_(self.h_off[s], non_blocking=True)
            if self.cuda_graph is not None:
                self.cuda_graph.replay()
            else:
                self._launch()
            if nr:
                self.h_new[s][:nr].copy_(self.d_new[:nr], non_blocking=True)
            self.done[s].record(self.stream)
        self.launches += 1

    def prepare(self):
        """Grow the graph's scratch to the capacity with one empty batch and,
        when requested, capture the insert as a CUDA graph."""
        torch = self.torch
        for h in self.h_off:
            h.zero_()
        with torch.cuda.stream(self.stream):
            self.d_off.zero_()
        # scratch sized for the capacity: one insert with the full hint
        self._launch()
        self.stream.synchronize()
        self.g.synchronize()
        if self.use_graph:
            cg = torch.cuda.CUDAGraph()
            with torch.cuda.graph(cg, stream=self.stream):
                self._launch()
            self.cuda_graph = cg
        return self

    def insert(self, batch, wait=True):
        """Insert one batch; returns its per-read new-k-mer counts (numpy) when
        wait, else None (the counts land in staging set 0 when done[0] fires)."""
        self.done[1].synchronize()     # a pipelined call may still use the GPU
        self.done[0].synchronize()
        self._fill(batch, 0)
        self._submit(batch, 0)
        if not wait:
            return None
        self.done[0].synchronize()
        return self.h_new[0][:batch.n_reads].numpy().view(np.uint64).copy()

    def insert_stream(self, reads):
        """Insert a whole PackedReads in capacity-sized batches, in order;
        returns the per-read new counts for all reads.  The host fills the
        next batch's staging set while the current batch is on the GPU."""
        out = np.zeros(reads.n_reads, np.uint64)
        bats = split_batches(reads, self.max_reads, self.max_bases)
        if not bats:
            return out
        self.done[0].synchronize()
        self.done[1].synchronize()
        self._fill(bats[0][1], 0)
        for i, (r0, b) in enumerate(bats):
            s = i & 1
            self._submit(b, s)
            if i + 1 < len(bats):
                # set s^1 was last used by batch i-1, finished below last round
                self._fill(bats[i + 1][1], s ^ 1)
            self.done[s].synchronize()
            out[r0:r0 + b.n_reads] = self.h_new[s][:b.n_reads].numpy().view(np.uint64)
        return out


# ---- autotuner --------------------------------------------------------------

def _cache_path():
    base = os.environ.get("GOETIA_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                                              "goetia_gb300"))
    return os.path.join(base, "autotune.json")


def _key(graph, max_reads, max_bases):
    st = type(graph).storage_type.__name__
    sh = type(graph).shifter_type.__name__
    cells = sum(graph.storage.tablesizes)
    return f"{st}/{sh}/K{graph.K}/n{len(graph.storage.tablesizes)}/c{cells.bit_length()}/" \
           f"r{int(max_reads).bit_length()}/b{int(max_bases).bit_length()}"


def candidates(storage_type, use_graph=True):
    """Schedules tried by the autotuner: the segmented bucketed path at its
    adaptive bucket size, the ordered bucketed path at three bucket sizes,
    the persistent fused hash+insert kernel at two claim windows, and --
    without graph replay -- the windowed path at two windows and two k-mers
    per thread."""
    from . import dbg as D
    fs0 = {D.BitStorage: 19, D.ByteStorage: 16, D.NibbleStorage: 17}[storage_type]
    out = [{"path": "bucketed", "bucket_bits": 0}]
    out += [{"path": "bucketed_ordered", "bucket_bits": fs} for fs in (fs0 - 1, fs0, fs0 + 1)]
    out += [{"path": "persistent", "window": w, "kpt": 4} for w in (262144, 1048576)]
    if not use_graph:
        out += [{"path": "windowed", "window": w, "kpt": k}
                for w in (262144, 1048576) for k in (4, 8)]
    return out


def apply_schedule(graph, sched):
    graph.set_insert_path(sched["path"])
    if sched["path"].startswith("bucketed"):
        graph.set_bucket_bits(sched["bucket_bits"])
        graph._bucket_bits = sched["bucket_bits"]
    else:
        graph.set_insert_schedule(sched.get("window", 0), sched.get("kpt", 0))


def autotune(graph, sample, max_reads, max_bases, repeats=2, use_cache=True, verbose=False,
             use_graph=True):
    """Pick the fastest schedule for inserting batches like `sample` (a
    PackedReads within the capacity) into tables shaped like `graph`'s.
    Timing runs on scratch clones; the choice is cached on disk per
    (storage, shifter, K, tables, capacity) and applied to `graph`."""
    key = _key(graph, max_reads, max_bases) + ("/graph" if use_graph else "")
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        apply_schedule(graph, cache[key]["schedule"])
        return cache[key]
    torch = __import__("torch")
    best = None
    trials = []
    for sched in candidates(type(graph).storage_type, use_graph):
        g = graph.clone()
        try:
            apply_schedule(g, sched)
            if sched["path"].startswith("bucketed") and not bucketed_fits(
                    g, max(max_bases - g.K + 1, 1), sched["bucket_bits"]):
                continue
            try:
                ins = BatchedInserter(g, max_reads, max_bases, use_graph=use_graph).prepare()
            except RuntimeError:
                continue                             # a launch the capture does not take
            ins.insert(sample)                       # warm state
            t = []
            for _ in range(repeats):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ins.insert(sample)
                t.append(time.perf_counter() - t0)
            sec = min(t)
        except _lib.GoetiaError:
            continue
        finally:
            del g
        trials.append({"schedule": sched, "seconds": sec})
        if verbose:
            print("autotune", sched, f"{sec * 1e3:.2f} ms")
        if best is None or sec < best["seconds"]:
            best = {"schedule": sched, "seconds": sec}
    best["trials"] = trials
    apply_schedule(graph, best["schedule"])
    if use_cache:
        cache[key] = best
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    return best


def autotune_capacity(graph, reads, capacities, use_graph=True, verbose=False):
    """Pick the batch capacity (reads, bases) -- the chunk size -- and, for it,
    the schedule, by timing the insert of the first batch of `reads` at each
    capacity on scratch clones.  Returns (capacity, best)."""
    best = None
    for cap in capacities:
        parts = split_batches(reads, cap[0], cap[1])
        if not parts:
            continue
        sample = parts[0][1]
        res = autotune(graph.clone(), sample, cap[0], cap[1], use_cache=False, verbose=verbose,
                       use_graph=use_graph)
        rate = sample.n_kmers(graph.K) / res["seconds"]
        if verbose:
            print("capacity", cap, f"{rate / 1e9:.2f} G k-mers/s")
        if best is None or rate > best[2]:
            best = (cap, res, rate)
    apply_schedule(graph, best[1]["schedule"])
    return best[0], best[1]
