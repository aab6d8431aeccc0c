"""Benchmark: k-mers inserted/s into dBG<ByteStorage, CanLemireShifter> on one GB300.

Workload (large count-min insert): K=31, 4 uint8 saturating tables of prime
size just below 2^30 cells (4 GiB, HBM-resident, far beyond the 129 MB L2),
reads of 150 bp sampled uniformly from either strand of a 50 Mbp seeded
random genome with 0.5% substitutions; 2% of reads carry an 'N' and are
dropped by the FASTX policy before packing.  One step inserts one batch of
1M reads (about 117M k-mers) in batch order with exact per-read new-k-mer
counts.  Tables persist across steps.

  value     k-mers/s with the batch already in HBM (device-pointer entry point)
  e2e       k-mers/s through the host-buffer C-ABI calls, H2D of the packed
            batch and D2H of the per-read new counts inside the timed region:
            gdbg_insert_batch_async (pipelined, the headline) and
            gdbg_insert_batch (returns with the counts, e2e.sync_call)
  plain     k-mers/s of the drop-in per-read insert_sequence call
  roofline  the insert path against the measured HBM copy bandwidth, with
            256 algorithmic bytes per k-mer (4 tables x 32 B sector, read +
            write)

``--impl reference`` times the reference algorithm on the host cores (the C
restatement in oracle/, all threads, shared tables) on the same workload.
Multi-GPU runs are independent replicas (the path does not shard here).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "k-mers inserted/s (K=31) plain vs batched/served on 1 GB300; p50/p99 chunk latency"
WORKLOAD = "large count-min insert: dBG<ByteStorage,CanLemireShifter> K=31, 4 x ~2^30 uint8 cells"
K = 31
N_TABLES = 4
MAX_TABLE = 1 << 30
READ_LEN = 150
GENOME_LEN = 50_000_000
SUB_RATE = 0.005
N_READ_FRAC = 0.02
BYTES_PER_KMER = 256    # 4 tables x 32 B sector x (read + write)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def over_ranks(dt, kmers, dev, world):
    """Whole-job figures of the replicas: the slowest rank's time and the
    k-mers all ranks inserted (each rank inserts its own batches)."""
    if world <= 1:
        return dt, float(kmers)
    import torch
    import torch.distributed as dist
    t = torch.tensor([dt], dtype=torch.float64, device=dev)
    k = torch.tensor([float(kmers)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(k)
    return float(t.item()), float(k.item())


def make_batches(n_batches, reads_per_step, seed0=4, native=True):
    """Seeded batches of packed reads (N-reads already dropped).  native=False
    packs with numpy alone, so the reference arm never loads the GPU library;
    both give the same words."""
    from goetia_gb300 import synth
    g = synth.genome(GENOME_LEN, 3)
    out = []
    for b in range(n_batches):
        rows = synth.sample_reads(g, reads_per_step, READ_LEN, SUB_RATE, seed0 + 1000 * b)
        keep = ~synth.n_read_mask(reads_per_step, N_READ_FRAC, seed0 + 1000 * b + 1)
        pr = synth.rows_to_packed(rows[keep], native=native)
        pr.n_skipped = int((~keep).sum())
        out.append(pr)
    return out


def oracle_check_headline(batches, sizes, gpu_tables, gpu_last_new, gpu_occupied, threads):
    """Bit-exact check of the timed run's end state against the oracle at the
    full benchmark shape (4 x ~2^30 Byte cells, every batch of the run).  The
    final table bytes do not depend on insertion order (a cell ends at
    min(255, its touches)), so all batches but the last go in with the
    oracle's multi-threaded insert; the last batch goes in sequentially, in
    batch order, which gives the reference's per-read new counts for it.
    Compared: those counts, all table bytes, and n_occupied (the non-zero
    cells of table 0).  A generator: the multi-threaded insert runs up to its
    yield, the rest when it is resumed (see run_checks)."""
    import oracle
    t0 = time.perf_counter()
    st = oracle.Storage("byte", sizes)
    for pr in batches[:-1]:
        st.insert_reads_mt(True, K, pr.packed, pr.offsets, threads)
    yield   # the multi-threaded part is done; the rest runs on one thread
    last = batches[-1]
    _, want_new = st.insert_reads(True, K, last.packed, last.offsets)
    new_ok = bool(np.array_equal(gpu_last_new, want_new))
    tables_ok = True
    step = 1 << 26
    for i, gt in enumerate(gpu_tables):
        ot = st.table_view(i)
        tables_ok &= len(ot) == len(gt)
        for a in range(0, len(gt), step):
            if not tables_ok:
                break
            tables_ok &= bool(np.array_equal(ot[a:a + step], gt[a:a + step]))
    occ_ok = int(np.count_nonzero(st.table_view(0))) == int(gpu_occupied)
    out = {"exact_vs_oracle": bool(new_ok and tables_ok and occ_ok),
           "last_batch_new_counts_equal": new_ok, "table_bytes_equal": bool(tables_ok),
           "n_occupied_equal": occ_ok,
           "checked": f"all {len(batches)} batches of the run ({sum(b.n_reads for b in batches)} "
                      f"reads) into 4 x ~2^30 oracle cells; per-read new counts of the last "
                      f"batch ({last.n_reads} reads, sequential oracle insert), all "
                      f"{sum(len(t) for t in gpu_tables)} table bytes, n_occupied",
           "seconds": time.perf_counter() - t0}
    del st
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic_per_kmer(name="insert_byte_k31_traffic.txt"):
    """DRAM bytes per k-mer from a committed ncu summary under profiles/ (its
    `dram_bytes_per_kmer=` line), or None."""
    p = os.path.join(HERE, "profiles", name)
    try:
        for ln in open(p):
            if ln.startswith("dram_bytes_per_kmer="):
                return float(ln.split("=", 1)[1])
    except OSError:
        pass
    return None


def cpu_baseline_port(batches, sample_reads, threads):
    """The oracle's C restatement on the host cores: one thread by default
    (the reference's execution model), on a bounded sample of the workload."""
    import oracle
    sizes = oracle.primes(N_TABLES, MAX_TABLE)
    st = oracle.Storage("byte", sizes)
    pr = batches[0]
    n = min(sample_reads, pr.n_reads)
    off = pr.offsets[:n + 1].copy()
    # warm the table pages with a small insert first
    warm = min(2000, n)
    st.insert_reads_mt(True, K, pr.packed, pr.offsets[:warm + 1].copy(), threads)
    t0 = time.perf_counter()
    if threads == 1:
        total, _ = st.insert_reads(True, K, pr.packed, off)
    else:
        total = st.insert_reads_mt(True, K, pr.packed, off, threads)
    dt = time.perf_counter() - t0
    return total / dt, total, dt


def run_serving(args, check_streams=3):
    """Config 5: 64 streams, each its own dBG<BitStorage, CanLemireShifter>
    (K=31, 4 tables of 2^24-2^28 bits, log-uniform per stream), stream sizes
    log-uniform in 10k-5M reads of 150 bp (times args.serve_scale, 1 by
    default) with 1% substitutions, arriving as 8-4096-read chunks on Poisson
    timing.  One full run at a mean gap of args.serve_gap per stream, then a
    sweep of arrival rates over a time window of the same streams
    (args.serve_window seconds of arrivals per rate), reporting p50/p99 chunk
    latency and aggregate k-mers/s at each; the capacity point is the highest
    swept rate whose p99 stays under 5 ms.  The check (run later) replays
    streams of the full run sequentially on the GPU and the smallest one on
    the oracle, chunk by chunk."""
    import goetia_gb300 as G
    from goetia_gb300 import serving
    sc = args.serve_scale
    cache = {}

    def specs_for(gap, window=None):
        return serving.make_streams(args.serve_streams, 17, reads_lo=max(8, int(10_000 * sc)),
                                    reads_hi=max(16, int(5_000_000 * sc)), chunk_lo=8,
                                    chunk_hi=4096, table_lo_bits=24, table_hi_bits=28,
                                    mean_gap_s=gap, genome_len=2_000_000, max_arrival_s=window,
                                    reads_cache=cache)

    def serve(specs):
        budget = int(args.serve_budget_gb * (1 << 30))
        if args.serve_loop == "python":
            srv = serving.Server(G.BitStorage, G.CanLemireShifter, K=31, n_tables=4,
                                 hbm_budget=budget, depth=4)
        else:
            srv = serving.NativeServer(G.BitStorage, G.CanLemireShifter, K=31, n_tables=4,
                                       hbm_budget=budget, depth=4,
                                       dispatch_threads=args.serve_dispatch_threads)
        return srv.run(specs)

    t0 = time.perf_counter()
    specs = specs_for(args.serve_gap)
    gen_s = time.perf_counter() - t0
    results, stats = serve(specs)
    offered = sum(sp.n_kmers(31) for sp in specs)
    sweep = []
    for gap in args.serve_sweep_gaps:
        sw_specs = specs_for(gap, args.serve_window)
        _, st = serve(sw_specs)
        sweep.append({"mean_gap_ms": gap * 1e3,
                      "offered_kmers_per_s": sum(sp.n_kmers(31) for sp in sw_specs) / args.serve_window,
                      "kmers_per_s": st["kmers_per_s"], "p50_ms": st["p50_ms"],
                      "p99_ms": st["p99_ms"], "chunks": st["chunks"]})
        del sw_specs
    ok = [x for x in sweep if x["p99_ms"] < 5.0]
    capacity = max(ok, key=lambda x: x["kmers_per_s"]) if ok else None
    out = {
        "streams": len(specs), "chunks": stats["chunks"],
        "reads": sum(sum(c.n_reads for c in sp.chunks) for sp in specs),
        "p50_chunk_latency_ms": stats["p50_ms"], "p99_chunk_latency_ms": stats["p99_ms"],
        "max_chunk_latency_ms": stats["max_ms"],
        "kmers_per_s": stats["kmers_per_s"], "kmers": stats["kmers"],
        "wall_s": stats["wall_s"], "offered_kmers": offered,
        "peak_hbm_GB": stats["peak_hbm_bytes"] / (1 << 30),
        "admission_waits": stats["admission_waits"], "lazy_frees": stats["lazy_frees"],
        "host": {k: v for k, v in stats.items() if k.startswith(("admit_", "dispatch_"))},
        "loop": (f"native runtime (gdbg_server_*), {args.serve_dispatch_threads} dispatcher "
                 "threads" if args.serve_loop == "native" else "Python loop (serving.Server)"),
        "hbm_budget_GB": args.serve_budget_gb,
        "rate_sweep": sweep,
        "capacity_at_p99_under_5ms": capacity,
        "generator_seconds": gen_s,
        "workload": (f"64 streams, reads 10k-5M x {sc} log-uniform, chunks 8-4096 reads, "
                     f"Poisson mean gap {args.serve_gap * 1e3:.1f} ms per stream, "
                     "Bit 4 x 2^24-2^28 bits per stream; sweep: "
                     f"{args.serve_window:.1f} s of arrivals per rate"),
    }
    by_size = sorted(specs, key=lambda sp: sum(c.n_reads for c in sp.chunks))
    replay_specs = [by_size[0], by_size[len(by_size) // 2], by_size[-1]][:check_streams]
    oracle_spec = by_size[0]
    served = {sp.sid: results[sp.sid] for sp in replay_specs + [oracle_spec]}
    del results, specs

    def check(threads):
        import oracle
        yield
        exact = True
        for sp in replay_specs:
            want = serving.replay(sp)
            exact &= all(np.array_equal(r.n_new, w) for r, w in zip(served[sp.sid], want))
        sizes = G.BitStorage.build(oracle_spec.max_table, 4).get_tablesizes()
        ref = oracle.Storage("bit", sizes)
        ok_or = True
        for r, c in zip(served[oracle_spec.sid], oracle_spec.chunks):
            _, want = ref.insert_reads(True, 31, c.packed, c.offsets)
            ok_or &= bool(np.array_equal(r.n_new, want))
        return {"exact_vs_sequential_replay": bool(exact),
                "replay_streams": [sum(c.n_reads for c in sp.chunks) for sp in replay_specs],
                "exact_vs_oracle": bool(ok_or),
                "oracle_stream_reads": sum(c.n_reads for c in oracle_spec.chunks)}

    return out, check


def masks_setup(n_reads):
    """Tables and query reads of the decision-mask workload: 4 x ~2^28-bit
    BitStorage (K=31) built from a 20 Mbp genome with 2,000 inserted 1-5 kb
    repeats and its 0.1% SNP haplotype; n_reads query reads of 150 bp sampled
    from both haplotypes, resident on cuda:0 with a mask buffer."""
    import numpy as np
    import torch
    import goetia_gb300 as G
    from goetia_gb300 import synth
    K = 31
    a, b = synth.repeat_genome(20_000_000, 2000, 1000, 5000, 0.001, 11)
    storage = G.BitStorage.build(1 << 28, 4)
    g = G.dBG[G.BitStorage, G.CanLemireShifter].build(storage, K)
    for hap in (a, b):
        g.insert_packed(synth.tiles_of(hap, 100_000, K))
    half = n_reads // 2
    q = np.concatenate([synth.sample_reads(a, half, 150, 0.0, 12),
                        synth.sample_reads(b, n_reads - half, 150, 0.0, 13)])
    pr = synth.rows_to_packed(q)
    dev = torch.device("cuda", 0)
    s = torch.cuda.Stream(dev)
    g.set_stream(s.cuda_stream)
    d_p = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
    d_o = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
    d_m = torch.empty(pr.n_kmers(K), dtype=torch.uint8, device=dev)
    return (a, b), storage, g, pr, s, d_p, d_o, d_m


def run_profile_masks(args):
    """The small case the decision-mask ncu captures run: the mask workload's
    own tables (4 x ~2^28 bits, 128 MiB) and args.mask_reads query reads,
    three mask passes."""
    from goetia_gb300 import build as gbuild
    gbuild.build()
    import torch
    _, _, g, pr, s, d_p, d_o, d_m = masks_setup(args.mask_reads)
    nk = pr.n_kmers(31)
    for rep in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        g.neighbor_masks_device(d_p.data_ptr(), d_p.numel(), d_o.data_ptr(), pr.n_reads,
                                d_m.data_ptr(), n_kmers=nk, stream=s.cuda_stream)
        e1.record(s)
        s.synchronize()
        ms = e0.elapsed_time(e1)
        print(json.dumps({"profile_masks_pass": rep, "kmers": nk, "ms": round(ms, 3),
                          "kmers_per_s": nk / (ms / 1000.0)}), flush=True)
    g.synchronize()
    return 0


def run_masks(args, check_reads=2000):
    """Config 4 shape: decision-node masks against a resident BitStorage, K=31.
    Tables (4 x ~2^28 bits) are built from a 20 Mbp genome with 2,000 inserted
    1-5 kb repeats and a 0.1% SNP haplotype; every k-mer of the query reads
    (150 bp, sampled from both haplotypes) gets its 8-bit neighbour mask.
    args.mask_reads query reads (the configuration's 5M by default)."""
    import numpy as np
    import torch
    import oracle
    from goetia_gb300 import synth
    K = 31
    n = args.mask_reads
    (a, b), storage, g, pr, s, d_p, d_o, d_m = masks_setup(n)
    nk = pr.n_kmers(K)
    for _ in range(2):
        g.neighbor_masks_device(d_p.data_ptr(), d_p.numel(), d_o.data_ptr(), pr.n_reads,
                                d_m.data_ptr(), n_kmers=nk, stream=s.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record(s)
    for _ in range(reps):
        g.neighbor_masks_device(d_p.data_ptr(), d_p.numel(), d_o.data_ptr(), pr.n_reads,
                                d_m.data_ptr(), n_kmers=nk, stream=s.cuda_stream)
    e1.record(s)
    s.synchronize()
    g.synchronize()
    dt = e0.elapsed_time(e1) / 1000.0 / reps
    masks = d_m.cpu().numpy()
    lo = np.unpackbits((masks & 15)[:, None], axis=1).sum(1)
    hi = np.unpackbits((masks >> 4)[:, None], axis=1).sum(1)
    sizes = storage.get_tablesizes()
    # the query reads are spread over the two haplotypes: check the first
    # reads of each half
    half = pr.n_reads // 2
    kofs = np.zeros(pr.n_reads + 1, np.int64)
    kofs[1:] = np.cumsum(np.maximum(np.diff(pr.offsets.astype(np.int64)) - (K - 1), 0))
    picks = [(0, min(check_reads // 2, half)), (half, half + min(check_reads // 2, pr.n_reads - half))]
    got = [masks[kofs[r0]:kofs[r1]].copy() for r0, r1 in picks]
    del d_m, d_p, d_o, g

    def check(threads):
        # bit-exact check of samples against the oracle's walker on tables
        # built from the same tiles (final Bit tables do not depend on order)
        ref = oracle.Storage("bit", sizes)
        for hap in (a, b):
            t = synth.tiles_of(hap, 100_000, K)
            ref.insert_reads_mt(True, K, t.packed, t.offsets, threads)
        yield
        ok = True
        for (r0, r1), gm in zip(picks, got):
            b0 = int(pr.offsets[r0])
            w0 = b0 // 16
            sub_off = (pr.offsets[r0:r1 + 1] - np.uint64(16 * w0)).astype(np.uint64)
            want = ref.decision_masks(True, K, np.ascontiguousarray(pr.packed[w0:]), sub_off)
            ok &= bool(np.array_equal(gm, want))
        return {"exact_vs_oracle": ok,
                "checked": f"neighbour masks of {sum(r1 - r0 for r0, r1 in picks)} query reads "
                           "(the first of each haplotype's half) against the oracle's walker"}
    peak, peak_kind = measured_peak()
    tpk = profile_traffic_per_kmer("decision_masks_bit_k31_ncu.md")
    roof = None
    if tpk:
        roof = {"bound": "hbm", "achieved": nk / dt * tpk / 1e9, "peak": peak, "unit": "GB/s",
                "frac": nk / dt * tpk / 1e9 / peak, "dram_bytes_per_kmer": tpk,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "bytes_source": "DRAM read + write bytes per k-mer of an ncu capture of k_masks "
                                "on 500,000 of this leg's query reads and its tables "
                                "(profiles/decision_masks_bit_k31_ncu.md), times k-mers/s",
                "probes_per_kmer": "32 counted (8 neighbours x 4 tables); 15.6 sectors loaded"}
    return {"kmers_per_s": nk / dt, "ms_per_pass": dt * 1e3, "kmers": nk,
            "decision_kmers": int(((lo > 1) | (hi > 1)).sum()), "roofline": roof,
            "workload": f"{n} reads x 150 bp vs Bit 4 x ~2^28 bits built from a 20 Mbp "
                        "genome + 2,000 1-5 kb repeats + 0.1% SNP haplotype"}, check


def run_batched(args, check_reads=2000, later_batch=4, cell_width=1 << 20):
    """Config 3: uneven-length batched insert into
    dBG<NibbleStorage, FwdLemireShifter>, K=21, 4 tables of ~2^28 cells.
    Reads: args.batched_reads (the configuration's 2M by default) with
    log-normal lengths (median 4 kb, sigma 1, clipped 200 bp-60 kb) from 5
    random 10 Mbp genomes at abundances 1:2:4:8:16, 4% substitutions, 2%
    insertions, 2% deletions, made by the multi-threaded generator before the
    timed region.  The whole stream goes through BatchedInserter.insert_stream:
    capacity-sized batches replayed from one captured CUDA graph with the
    autotuned capacity and schedule, the host staging of the next batch
    overlapped with the current one; wall clock around the whole stream.  The
    plain per-read call is timed on 40 of the same reads.

    Returns (stats, check): `check` runs the oracle comparisons later (they
    take the host cores): the first check_reads reads from empty tables, the
    first check_reads reads of batch `later_batch` after an oracle fed the
    batches before it, and the final value of cell_width cells of tables 0
    and 3 after the whole stream (min(15, the oracle's touch count))."""
    import goetia_gb300 as G
    from goetia_gb300 import batched, synth
    import torch
    K = 21
    gens = [synth.genome(10_000_000, 5 + i) for i in range(5)]
    t0 = time.perf_counter()
    reads = synth.uneven_stream(gens, [1, 2, 4, 8, 16], args.batched_reads, 4000, 1.0, 200, 60_000,
                                0.04, 0.02, 0.02, 10)
    gen_s = time.perf_counter() - t0
    nk = reads.n_kmers(K)
    storage = G.NibbleStorage.build(1 << 28, 4)
    g = G.dBG[G.NibbleStorage, G.FwdLemireShifter].build(storage, K)
    caps = [(8192, 64 << 20), (16384, 128 << 20), (32768, 256 << 20)]
    cap, tuned = batched.autotune_capacity(g, reads, caps)
    ins = batched.BatchedInserter(g, cap[0], cap[1], use_graph=True).prepare()
    bat = batched.split_batches(reads, cap[0], cap[1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_new = ins.insert_stream(reads)   # host staging of the next batch overlapped
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    g.synchronize()
    sizes = storage.get_tablesizes()
    # the GPU's final cells of tables 0 and 3 in the checked ranges
    raw = g.get_raw()
    lo = [sizes[0] // 2, sizes[3] // 3]
    gpu_cells = []
    for ti, l in zip((0, 3), lo):
        c = np.arange(l, l + cell_width, dtype=np.int64)
        b = raw[ti][c // 2]
        gpu_cells.append(np.where(c % 2 == 0, b >> 4, b & 15).astype(np.uint8))
    del raw
    lb = min(later_batch, len(bat) - 1)

    # plain: one insert_sequence call per read on a fresh graph
    gp = g.clone()
    from goetia_gb300.reads import codes_to_str
    first = bat[0][1]
    n_plain = min(40, first.n_reads)
    j_all = np.arange(int(first.offsets[n_plain]))
    codes = ((first.packed[j_all >> 4] >> (2 * (j_all & 15)).astype(np.uint32)) & 3).astype(np.uint8)
    sample = [codes_to_str(codes[int(first.offsets[r]):int(first.offsets[r + 1])]).encode()
              for r in range(n_plain)]
    gp.insert_sequence(sample[0])
    t1 = time.perf_counter()
    pk = 0
    for sq in sample[1:]:
        pk += gp.insert_sequence(sq)
    plain = pk / (time.perf_counter() - t1)
    del gp
    peak, peak_kind = measured_peak()
    achieved = nk / dt * BYTES_PER_KMER / 1e9
    stats = {"kmers_per_s": nk / dt, "kmers": nk, "reads": reads.n_reads, "bases": reads.n_bases,
             "seconds": dt, "batches": len(bat), "capacity_reads_bases": list(cap),
             "schedule": tuned["schedule"], "cuda_graph": ins.cuda_graph is not None,
             "autotune_trials_ms": [{**t["schedule"], "ms": round(1e3 * t["seconds"], 3)}
                                    for t in tuned.get("trials", [])],
             "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "algorithmic_bytes_per_kmer": BYTES_PER_KMER,
                          "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
             "generator_seconds": gen_s,
             "plain_kmers_per_s": plain, "batched_over_plain": (nk / dt) / plain,
             "workload": f"{reads.n_reads} uneven reads (log-normal, median 4 kb, sigma 1, "
                         "200 bp-60 kb), 5 x 10 Mbp genomes 1:2:4:8:16, 4% sub / 2% ins / 2% del; "
                         "Nibble 4 x ~2^28 cells, FwdLemireShifter, K=21"}
    del ins, g

    def check(threads):
        import oracle
        t = time.perf_counter()
        out = {}
        # multi-threaded part: the batches before the later batch (final
        # cells do not depend on order), and the touch counts of the checked
        # cells over the whole stream
        ref_later = oracle.Storage("nibble", sizes)
        for r0, b in bat[:lb]:
            ref_later.insert_reads_mt(False, K, b.packed, b.offsets, threads)
        cnt = oracle.count_cells(False, K, reads.packed, reads.offsets, sizes, [0, 3], lo,
                                 cell_width, threads=threads)
        yield
        # (1) the first reads from empty tables, in batch order
        b0 = bat[0][1]
        sub = G.PackedReads(b0.packed, b0.offsets[:min(check_reads, b0.n_reads) + 1].copy())
        ref = oracle.Storage("nibble", sizes)
        _, want = ref.insert_reads(False, K, sub.packed, sub.offsets)
        out["first_reads_new_counts_equal"] = bool(np.array_equal(n_new[:sub.n_reads], want))
        del ref
        # (2) the first reads of the later batch, in order, after its prefix
        r0, b = bat[lb]
        sub = G.PackedReads(b.packed, b.offsets[:min(check_reads, b.n_reads) + 1].copy())
        _, want = ref_later.insert_reads(False, K, sub.packed, sub.offsets)
        out["later_batch_new_counts_equal"] = bool(np.array_equal(n_new[r0:r0 + sub.n_reads], want))
        del ref_later
        # (3) final cells after the whole stream
        out["final_cells_equal"] = bool(all(np.array_equal(gpu_cells[j], np.minimum(cnt[j], 15))
                                            for j in range(2)))
        out["exact_vs_oracle"] = bool(out["first_reads_new_counts_equal"] and
                                      out["later_batch_new_counts_equal"] and
                                      out["final_cells_equal"])
        out["checked"] = (f"per-read new counts of the first {check_reads} reads (empty tables) "
                          f"and of the first {check_reads} reads of batch {lb} (oracle fed "
                          f"batches 0-{lb - 1}); final values of {cell_width} cells of tables "
                          f"0 and 3 after all {reads.n_reads} reads")
        out["seconds"] = time.perf_counter() - t
        return out

    return stats, check


def run_fastx(args, n_reads, seed):
    """FASTQ text of one benchmark batch (the same seeded reads; each read
    the generator marks for an 'N' gets one), parsed and packed on the GPU
    by gdbg_parse_fastx_device (FastxParser<DNA_SIMPLE>::next over kseq,
    then the packer's policy).  Timed with CUDA events over whole calls
    (text already in HBM); checked against the batch the benchmark packs
    from the same reads: packed words, offsets and dropped reads."""
    import torch
    from goetia_gb300 import synth, reads as R
    g = synth.genome(GENOME_LEN, 3)
    rows = synth.sample_reads(g, n_reads, READ_LEN, SUB_RATE, seed)
    keep = ~synth.n_read_mask(n_reads, N_READ_FRAC, seed + 1)
    seq = np.frombuffer(b"ACGT", np.uint8)[rows]
    idx = np.nonzero(~keep)[0]
    seq[idx, (idx * 37) % READ_LEN] = ord("N")
    head = np.empty((n_reads, 10), np.uint8)
    head[:, 0], head[:, 1], head[:, 9] = ord("@"), ord("r"), ord("\n")
    i = np.arange(n_reads)
    for d in range(7):
        head[:, 2 + d] = (i // 10 ** (6 - d)) % 10 + ord("0")
    nl = np.full((n_reads, 1), ord("\n"), np.uint8)
    plus = np.tile(np.frombuffer(b"+\n", np.uint8), (n_reads, 1))
    qual = np.full((n_reads, READ_LEN), ord("I"), np.uint8)
    text = np.ascontiguousarray(np.concatenate([head, seq, nl, plus, qual, nl], axis=1)).reshape(-1)
    expect = synth.rows_to_packed(rows[keep])
    dev = torch.device("cuda", 0)
    d_text = torch.from_numpy(text).to(dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    for _ in range(2):
        packed, offsets, st = R.parse_fastx_device(d_text, stream=stream.cuda_stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    torch.cuda.synchronize(dev)
    ev0.record(stream)
    for _ in range(reps):
        packed, offsets, st = R.parse_fastx_device(d_text, stream=stream.cuda_stream)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    off = offsets.cpu().numpy().view(np.uint64)
    nw = (int(off[-1]) + 15) // 16
    exact = (st["n_kept"] == expect.n_reads and st["n_dropped"] == int((~keep).sum()) and
             np.array_equal(off, expect.offsets) and
             np.array_equal(packed.cpu().numpy().view(np.uint32)[:nw], expect.packed[:nw]))
    del d_text, packed, offsets
    torch.cuda.empty_cache()
    return {"text_GB_per_s": text.size / ms / 1e6, "reads_per_s": n_reads / ms * 1e3,
            "ms_per_call": ms, "text_bytes": int(text.size), "reads": n_reads,
            "reads_kept": st["n_kept"], "reads_dropped": st["n_dropped"],
            "exact_vs_host_packed_batch": bool(exact),
            "workload": f"FASTQ text of one benchmark batch ({n_reads} reads x {READ_LEN} bp, "
                        "four-line records, N-reads dropped), in HBM; one "
                        "gdbg_parse_fastx_device call (count, lines, classify, gather, pack)"}


def run_profile_case(args):
    """The small case the ncu captures run: dBG<ByteStorage, CanLemireShifter>,
    K=31, 4 x ~2^28 cells (1 GiB of tables, 8x L2) through the segmented path,
    three batches of 250,000 reads x 150 bp from a 20 Mbp seeded genome with
    0.5% substitutions -- the benchmark's tables-to-batch ratio (36 table bytes
    per k-mer) at a quarter of its size.  The batches are inserted from device
    buffers, like the benchmark's timed steps, so each kernel is one launch
    per batch."""
    import torch
    import goetia_gb300 as G
    from goetia_gb300 import build as gbuild, synth
    gbuild.build()
    dev = torch.device("cuda", 0)
    gen = synth.genome(20_000_000, 3)
    g = G.dBG[G.ByteStorage, G.CanLemireShifter].build(G.ByteStorage.build(1 << 28, 4), K)
    g.set_insert_path("bucketed")
    stream = torch.cuda.Stream(dev)
    g.set_stream(stream.cuda_stream)
    for b in range(3):
        pr = synth.rows_to_packed(synth.sample_reads(gen, 250_000, READ_LEN, SUB_RATE, 10 + b))
        d_packed = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
        d_off = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
        d_new = torch.empty(pr.n_reads, dtype=torch.int64, device=dev)
        torch.cuda.synchronize(dev)
        g.insert_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), pr.n_reads,
                        n_kmers=pr.n_kmers(K), n_new_ptr=d_new.data_ptr(),
                        stream=stream.cuda_stream)
        g.synchronize()
        print(json.dumps({"profile_case_batch": b, "kmers": pr.n_kmers(K),
                          "new_kmers": int(d_new.sum().item())}), flush=True)
    return 0


def run_reference(args):
    """The reference's insert algorithm on the host cores: the oracle's C
    restatement (the reference's own objects are x86 builds that do not run
    on the Arm GPU host), all threads sharing one storage, over the same
    warm-up + timed batches the GPU arm inserts (same seeds, generated and
    packed with numpy alone), into the same 4 x ~2^30-cell Byte tables."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    threads = os.cpu_count() or 1
    batches = make_batches(args.warmup + args.steps, args.reads_per_step, native=False)
    sizes = oracle.primes(N_TABLES, MAX_TABLE)
    st = oracle.Storage("byte", sizes)
    for pr in batches[:args.warmup]:
        st.insert_reads_mt(True, K, pr.packed, pr.offsets, threads)
    t0 = time.perf_counter()
    total = 0
    for pr in batches[args.warmup:]:
        total += st.insert_reads_mt(True, K, pr.packed, pr.offsets, threads)
    dt = time.perf_counter() - t0
    v = total / dt
    n = batches[0].n_reads
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "k-mers/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64/u8",
        "data": "synthetic (seeded genome and reads)",
        "config": {"workload": WORKLOAD, "reads_per_step": int(n), "read_len": READ_LEN,
                   "table_cells": sizes, "genome_bp": GENOME_LEN, "substitution_rate": SUB_RATE,
                   "batches": f"the GPU arm's {args.warmup} warm-up + {args.steps} timed "
                              "batches, same seeds"},
        "cpu_baseline": {"value": v, "unit": "k-mers/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} distinct batches of ~{n} reads x {READ_LEN} bp "
                                   f"({total} k-mers), C restatement of the reference insert, "
                                   f"{threads} threads on one shared storage"},
        "e2e": {"value": v, "unit": "k-mers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "repo_libraries_loaded": repo_libraries_loaded(),
    }
    print(json.dumps(line), flush=True)
    return 0


def repo_libraries_loaded():
    """Shared objects of this repository mapped into the process (Linux)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return []
    return sorted(os.path.relpath(p, HERE) for p in paths if p.startswith(HERE + os.sep))


def run_checks(checks):
    """Run the legs' oracle checks on the host cores.  Each check is a
    generator function of a thread count: its multi-threaded part runs up to
    its yield (one check after another, each with all cores), then the
    single-threaded remainders run side by side (ctypes releases the GIL).
    Returns {leg: result}; a check that raises reports the error, never hides
    it."""
    out, pending = {}, {}
    cores = max(1, (os.cpu_count() or 2) - 1)
    for name, fn in checks.items():
        try:
            gen = fn(cores)
            next(gen)
            pending[name] = gen
        except StopIteration as e:
            out[name] = e.value
        except Exception as e:
            out[name] = {"exact_vs_oracle": False, "error": repr(e)}

    def finish(name, gen):
        try:
            next(gen)
            out[name] = {"exact_vs_oracle": False, "error": "check did not finish"}
        except StopIteration as e:
            out[name] = e.value
        except Exception as e:
            out[name] = {"exact_vs_oracle": False, "error": repr(e)}

    th = [threading.Thread(target=finish, args=kv, daemon=True) for kv in pending.items()]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return out


def run_gpu(args):
    import torch
    import goetia_gb300 as G
    from goetia_gb300 import build as gbuild

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    gbuild.build()
    dev = torch.device("cuda", local)

    n_batches = args.warmup + args.steps
    batches = make_batches(n_batches, args.reads_per_step, seed0=4 + 7919 * rank)

    storage = G.ByteStorage.build(MAX_TABLE, N_TABLES)
    Graph = G.dBG[G.ByteStorage, G.CanLemireShifter]
    g = Graph.build(storage, K)
    if args.window:
        g.set_insert_schedule(args.window, args.kpt)
    stream = torch.cuda.Stream(dev)
    g.set_stream(stream.cuda_stream)

    # device-resident inputs
    d_batches = []
    for pr in batches:
        d_packed = torch.from_numpy(pr.packed.view(np.int32)).to(dev)
        d_off = torch.from_numpy(pr.offsets.view(np.int64)).to(dev)
        d_new = torch.empty(pr.n_reads, dtype=torch.int64, device=dev)
        d_batches.append((d_packed, d_off, d_new, pr.n_reads, pr.n_kmers(K)))
    torch.cuda.synchronize(dev)

    def step_on(graph, i):
        d_packed, d_off, d_new, n_reads, nk = d_batches[i]
        graph.insert_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), n_reads,
                            n_kmers=nk, n_new_ptr=d_new.data_ptr(), stream=stream.cuda_stream)
        return nk

    def step(i):
        return step_on(g, i)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()

    g.stage_times()   # reset the stage totals
    launches0 = g.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kmers = 0
    with ClockSampler(local) as clocks:
        time.sleep(0.3)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for i in range(args.warmup, n_batches):
            kmers += step(i)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        time.sleep(0.1)
    launches = g.launch_count() - launches0
    g.synchronize()   # raises if a device-side check fired
    dt = e0.elapsed_time(e1) / 1000.0
    # per-stage times of the same steps, measured with CUDA events on the
    # launching stream in a second timed pass over the same batches on a clone
    g_prof = g.clone()
    g_prof.set_stream(stream.cuda_stream)
    g_prof.set_profiling(True)
    for i in range(args.warmup):
        step_on(g_prof, i)
    torch.cuda.synchronize(dev)
    g_prof.stage_times()
    for i in range(args.warmup, n_batches):
        step_on(g_prof, i)
    torch.cuda.synchronize(dev)
    stages = g_prof.stage_times()
    del g_prof
    dt, total_kmers = over_ranks(dt, kmers, dev, world)
    value = total_kmers / dt

    # e2e: host-buffer C-ABI calls on fresh graphs, copies inside the timed region
    pinned = []
    for pr in batches:
        hp = torch.from_numpy(pr.packed.view(np.int32)).pin_memory().numpy().view(np.uint32)
        ho = torch.from_numpy(pr.offsets.view(np.int64)).pin_memory().numpy().view(np.uint64)
        hn = torch.empty(max(pr.n_reads, 1), dtype=torch.int64).pin_memory().numpy().view(np.uint64)
        pinned.append((G.PackedReads(hp, ho), hn))
    import ctypes
    from goetia_gb300 import _lib

    def sync_step(gx, i):
        # gdbg_insert_batch: returns when the counts are in host memory
        pr, hn = pinned[i]
        nk = _lib.c_u64()
        _lib.call("gdbg_insert_batch", gx._h, pr.packed.ctypes.data_as(_lib.u32p), pr.packed.size,
                  pr.offsets.ctypes.data_as(_lib.u64p), pr.n_reads, hn.ctypes.data_as(_lib.u64p),
                  ctypes.byref(nk))
        return int(nk.value)

    def async_step(gx, i):
        # gdbg_insert_batch_async: queued on the graph's stream, the copies of
        # large batches on its second stream, overlapping the batch before
        # (the call counts the batch's k-mers from the host offsets)
        pr, hn = pinned[i]
        gx.insert_async(pr.packed.ctypes.data, pr.packed.size, pr.offsets.ctypes.data, pr.n_reads,
                        None, hn.ctypes.data)
        return batch_kmers[i]

    # k-mers per batch for the throughput figure (outside the timed region)
    batch_kmers = [int(np.maximum(np.diff(pr.offsets.view(np.int64)) - (K - 1), 0).sum())
                   for pr in batches]

    def e2e_run(step):
        gx = g.clone()
        if args.window:
            gx.set_insert_schedule(args.window, args.kpt)
        for i in range(args.warmup):
            step(gx, i)
        gx.synchronize()
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        kmers = h2d = d2h = 0
        for i in range(args.warmup, n_batches):
            kmers += step(gx, i)
            pr = pinned[i][0]
            h2d += pr.packed.nbytes + pr.offsets.nbytes
            d2h += pr.n_reads * 8
        gx.synchronize()
        torch.cuda.synchronize(dev)
        dt = time.perf_counter() - t0
        dt, total = over_ranks(dt, kmers, dev, world)
        # parity spot check against the device-resident arm: same batches into
        # fresh tables, so the last batch's per-read new counts agree
        same = bool(np.array_equal(pinned[-1][1][:batches[-1].n_reads],
                                   d_batches[-1][2].cpu().numpy().view(np.uint64)))
        del gx
        return total / dt, h2d, d2h, same

    sync_value, _, _, sync_same = e2e_run(sync_step)
    e2e_value, h2d, d2h, same = e2e_run(async_step)
    same = same and sync_same

    # plain drop-in: one insert_sequence call per read
    from goetia_gb300.reads import codes_to_str
    g3 = g.clone()
    pr0 = batches[0]
    n_plain = min(args.plain_reads, pr0.n_reads)
    j = np.arange(int(pr0.offsets[n_plain]))
    codes = ((pr0.packed[j >> 4] >> (2 * (j & 15)).astype(np.uint32)) & 3).astype(np.uint8)
    seqs = [codes_to_str(codes[int(pr0.offsets[r]):int(pr0.offsets[r + 1])]).encode()
            for r in range(n_plain)]
    for s in seqs[:20]:
        g3.insert_sequence(s)
    t0 = time.perf_counter()
    pk = 0
    for s in seqs[20:]:
        pk += g3.insert_sequence(s)
    plain_dt = time.perf_counter() - t0
    plain_value = pk / plain_dt

    # the timed run's end state, for the oracle check after the timed legs
    gpu_state = None
    if rank == 0 and not args.no_oracle_check:
        gpu_state = (g.get_raw(), d_batches[-1][2].cpu().numpy().view(np.uint64)[:batches[-1].n_reads],
                     g.n_occupied())

    peak, peak_kind = measured_peak()
    achieved = value / world * BYTES_PER_KMER / 1e9
    tpk = profile_traffic_per_kmer()
    per_step_kmers = kmers / max(args.steps, 1)
    stage_total = sum(ms for ms, _ in stages.values()) or 1.0
    dom_name, (dom_ms, dom_n) = max(stages.items(), key=lambda kv: kv[1][0]) if stages else ("", (0.0, 1))
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
        "kernel": "batch insert step: the k-mer insert pipeline of one batch",
        "algorithmic_bytes_per_kmer": BYTES_PER_KMER,
        "traffic": (tpk * per_step_kmers) if tpk else None,
        "traffic_unit": "DRAM bytes per step (ncu capture, scaled by k-mers)" if tpk else None,
        "dominant_kernel": {"name": dom_name, "share": dom_ms / stage_total,
                            "ms_per_launch": dom_ms / max(dom_n, 1), "launches": dom_n},
        "stages_ms_per_step": {k: v[0] / max(args.steps, 1) for k, v in stages.items()},
    }

    # the other configurations' legs; each returns its stats and a check that
    # runs the oracle comparisons after every timed leg is done
    checks = {}
    batched_stats = None
    if not args.no_batched:
        batched_stats, checks["batched_uneven"] = run_batched(args)
    mask_stats = None
    if not args.no_masks:
        mask_stats, checks["decision_masks"] = run_masks(args)
    fastx_stats = None
    if not args.no_fastx:
        fastx_stats = run_fastx(args, args.reads_per_step, 4 + 7919 * rank)
    serving_stats = None
    if not args.no_serving:
        del g, g3
        torch.cuda.empty_cache()
        serving_stats, checks["serving"] = run_serving(args)
    if gpu_state is not None:
        checks["headline"] = lambda threads: oracle_check_headline(
            batches, storage.get_tablesizes(), *gpu_state, threads)
    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            # timed alone, before the checks take the host cores
            v, tot, cdt = cpu_baseline_port(batches, args.cpu_sample_reads, 1)
            cpu = {"value": v, "unit": "k-mers/s", "cores": 1, "kind": "port",
                   "sample": f"{min(args.cpu_sample_reads, batches[0].n_reads)} reads x "
                             f"{READ_LEN} bp of step 0 ({tot} k-mers, {cdt:.1f} s), one thread, "
                             "4 x ~2^30-cell Byte tables"}
        exact = run_checks(checks)
        if batched_stats is not None:
            batched_stats["oracle_check"] = exact.get("batched_uneven")
        if mask_stats is not None:
            mask_stats["oracle_check"] = exact.get("decision_masks")
        if serving_stats is not None:
            serving_stats["oracle_check"] = exact.get("serving")
        exact = exact.get("headline", {})
        line = {
            "metric": METRIC, "value": value, "unit": "k-mers/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64/u8", "data": "synthetic (seeded genome and reads)",
            "config": {"workload": WORKLOAD, "storage": "ByteStorage",
                       "shifter": "CanLemireShifter", "K": K, "n_tables": N_TABLES,
                       "table_cells": storage.get_tablesizes(),
                       "reads_per_step": int(batches[0].n_reads), "read_len": READ_LEN,
                       "genome_bp": GENOME_LEN, "substitution_rate": SUB_RATE,
                       "n_reads_dropped_per_step": int(batches[0].n_skipped),
                       "insert_path": ("bucketed (segmented)" if "k_sp_apply" in stages else
                                       "bucketed (ordered)" if "k_bkt_apply" in stages else
                                       "windowed"),
                       "l2": "inputs larger than L2: 4 GiB of tables, random cells",
                       "exact_vs_oracle": exact.get("exact_vs_oracle"),
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "k-mers/s", "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps, "same_new_counts_as_value_arm": same,
                    "api": "gdbg_insert_batch_async from pinned host buffers, one call per batch, "
                           "per-read new counts copied back by each call",
                    "sync_call": {"value": sync_value, "unit": "k-mers/s",
                                  "api": "gdbg_insert_batch, returns with the counts in host memory"}},
            "plain": {"value": plain_value, "unit": "k-mers/s",
                      "sample": f"{n_plain - 20} reads, one insert_sequence call each"},
            "gpu_launches": int(launches),
            "serving": serving_stats,
            "decision_masks": mask_stats,
            "batched_uneven": batched_stats,
            "fastx_parse": fastx_stats,
            "roofline": roofline,
            "oracle_check": exact or None,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--reads-per-step", type=int, default=1_000_000)
    ap.add_argument("--window", type=int, default=0)
    ap.add_argument("--kpt", type=int, default=0)
    ap.add_argument("--plain-reads", type=int, default=2000)
    ap.add_argument("--cpu-sample-reads", type=int, default=300_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-masks", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-fastx", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true",
                    help="skip the oracle check of the timed run's end state")
    ap.add_argument("--batched-reads", type=int, default=2_000_000)
    ap.add_argument("--mask-reads", type=int, default=5_000_000)
    ap.add_argument("--serve-streams", type=int, default=64)
    ap.add_argument("--serve-scale", type=float, default=1.0)
    ap.add_argument("--serve-loop", default="native", choices=["native", "python"])
    ap.add_argument("--serve-dispatch-threads", type=int, default=4)
    ap.add_argument("--serve-window", type=float, default=3.0,
                    help="seconds of arrivals per point of the rate sweep")
    ap.add_argument("--serve-sweep-gaps", type=lambda v: [float(x) for x in v.split(",")],
                    default=[0.004, 0.002, 0.001, 0.0008, 0.00067, 0.00057, 0.0005, 0.00025],
                    help="mean chunk gaps per stream (s) of the rate sweep")
    ap.add_argument("--serve-gap", type=float, default=0.002)
    ap.add_argument("--serve-budget-gb", type=float, default=32.0)
    ap.add_argument("--profile-case", action="store_true",
                    help="run only the small insert case the ncu captures profile")
    ap.add_argument("--profile-fastx", action="store_true",
                    help="run only the FASTQ parse leg (one benchmark batch as text)")
    ap.add_argument("--profile-masks", action="store_true",
                    help="run only the decision-mask case the ncu captures profile "
                         "(--mask-reads query reads)")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args)
    if args.profile_fastx:
        from goetia_gb300 import build as gbuild
        gbuild.build()
        print(json.dumps(run_fastx(args, args.reads_per_step, 4)), flush=True)
        return 0
    if args.profile_masks:
        return run_profile_masks(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
