"""GPU parity: the CUDA path against the reference's golden fixtures and the
oracle, bit-exact (hashes, per-read new counts, table bytes, counts, masks,
n_unique / n_occupied).  Every check here goes through libgoetia_gb300.so."""
import numpy as np
import pytest

import oracle
from goldens import Case, names
import goetia_gb300 as G
from goetia_gb300 import synth

pytestmark = pytest.mark.gpu

STORAGES = {"bit": G.BitStorage, "byte": G.ByteStorage, "nibble": G.NibbleStorage}
SHIFTERS = {True: G.CanLemireShifter, False: G.FwdLemireShifter}


def graph_for(kind, canonical, K, sizes):
    st = STORAGES[kind](tablesizes=[int(s) for s in sizes])
    return G.dBG[STORAGES[kind], SHIFTERS[canonical]].build(st, K)


def check_tables(g, tables):
    got = g.get_raw()
    assert len(got) == len(tables)
    for a, b in zip(got, tables):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", names())
def test_golden_plain_per_read(cuda_ready, name):
    """insert_sequence per read (the drop-in, one call per read)."""
    c = Case(name)
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    for r, s in enumerate(c.reads):
        if len(s) < c.K:
            with pytest.raises(G.SequenceLengthException):
                g.insert_sequence_new(s)
            assert c.n_new[r] == 0
            continue
        nk, nn = g.insert_sequence_new(s)
        assert nk == int(c.n_kmers[r])
        assert nn == int(c.n_new[r]), (r, nn, int(c.n_new[r]))
    check_tables(g, c.tables)
    assert (g.n_unique(), g.n_occupied()) == (c.n_unique, c.n_occupied)
    k = 0
    for s in c.reads:
        if len(s) < c.K:
            continue
        n = len(s) - c.K + 1
        assert g.query_sequence(s) == [int(x) for x in c.counts[k:k + n]]
        val, fw, rc = g.hash_array(s)
        assert np.array_equal(val, c.val[k:k + n])
        if c.canonical:
            assert np.array_equal(fw, c.fw[k:k + n]) and np.array_equal(rc, c.rc[k:k + n])
        assert np.array_equal(g.neighbor_masks(s), c.masks[k:k + n])
        k += n


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
@pytest.mark.parametrize("K,lengths", [(31, [40, 600, 2500]), (101, [150, 1300]), (300, [320, 900])])
def test_plain_long_reads_vs_oracle(cuda_ready, kind, K, lengths):
    """insert_sequence on reads of several 512-k-mer chunks (the one-CTA read
    insert works through a read's k-mers chunk by chunk, in order) and of
    k-mers too long for its staged bases (K=300), on small tables so cells
    collide within a read: per-read new counts, tables and counters against
    the oracle's sequential insert."""
    from goetia_gb300 import reads as R
    sizes = oracle.primes(4, 50_000)
    g = graph_for(kind, True, K, sizes)
    ref = oracle.Storage(kind, sizes)
    gen = synth.genome(20_000, 71)
    rng = np.random.default_rng(72)
    rows = []
    for L in lengths * 3:
        s0 = int(rng.integers(0, len(gen) - L))
        rows.append(gen[s0:s0 + L].copy())
    pr = R.from_codes(rows)
    _, want = ref.insert_reads(True, K, pr.packed, pr.offsets)
    for r, codes in enumerate(rows):
        nk, nn = g.insert_sequence_new(R.codes_to_str(codes))
        assert nk == len(codes) - K + 1
        assert nn == int(want[r]), (r, nn, int(want[r]))
    check_tables(g, ref.tables())
    assert (g.n_unique(), g.n_occupied()) == ref.stats()


# insert path, window, k-mers per thread, log2 cells per bucket (0 = default)
PATHS = [("persistent", 262144, 4, 0), ("persistent", 64, 8, 0), ("persistent", 5, 4, 0),
         ("windowed", 262144, 4, 0), ("windowed", 64, 8, 0), ("windowed", 5, 4, 0),
         ("bucketed", 0, 0, 0), ("bucketed", 0, 0, 5), ("bucketed", 0, 0, 7),
         ("bucketed_ordered", 0, 0, 0), ("bucketed_ordered", 0, 0, 5)]


@pytest.mark.parametrize("name", names())
@pytest.mark.parametrize("path,window,kpt,fs", PATHS)
def test_golden_batched(cuda_ready, name, path, window, kpt, fs):
    """One packed batch through each insert path.  Windows smaller than the
    batch exercise the cross-window first-touch logic (and, at 32 k-mers per
    window, the claims epoch wrap after 127 windows); default buckets hold
    several 1024-record chunks, tiny buckets give many buckets and two digit
    passes."""
    c = Case(name)
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    g.set_insert_schedule(window, kpt)
    g.set_insert_path(path)
    if fs:
        g.set_bucket_bits(max(fs, 5) if c.storage == "bit" else fs)
    packed, off = c.packed()
    pr = G.PackedReads(packed, off)
    n_new = g.insert_packed(pr)
    assert np.array_equal(n_new, c.n_new)
    check_tables(g, c.tables)
    assert (g.n_unique(), g.n_occupied()) == (c.n_unique, c.n_occupied)
    assert np.array_equal(g.query_packed(pr), c.counts)
    val, fw, rc = g.hashes_packed(pr)
    assert np.array_equal(val, c.val)
    if c.canonical:
        assert np.array_equal(fw, c.fw) and np.array_equal(rc, c.rc)
    masks = g.neighbor_masks_packed(pr)
    assert np.array_equal(masks, c.masks)
    assert c.decision_positions(masks) == c.dpos


def test_known_answer_k27(cuda_ready):
    g = graph_for("bit", True, 27, [1009, 1013])
    h = g.hash("TCACCTGTGTTGTGCTACTTGCGGCGC")
    assert h.fw_hash == 13194817695400542713 and h.rc_hash == 4324216031038051805
    assert int(h) == 4324216031038051805
    # symbols past K are ignored (tests/test_dbg.py:124-127)
    assert int(g.hash("A" * 27)) == int(g.hash("A" * 27 + "TTTT"))


def _oracle_run(kind, canonical, K, sizes, pr):
    st = oracle.Storage(kind, sizes)
    total, n_new = st.insert_reads(canonical, K, pr.packed, pr.offsets)
    return st, n_new


@pytest.mark.parametrize("kind,canonical,K,max_table", [
    ("bit", True, 31, 1 << 22),       # config 1 shape: 4 Bloom tables of ~2^22 bits
    ("byte", True, 31, 50021),
    ("nibble", False, 21, 40009),
    ("bit", False, 25, 7919),
])
@pytest.mark.parametrize("path,fs", [("persistent", 0), ("windowed", 0), ("bucketed", 0),
                                     ("bucketed", 5), ("bucketed_ordered", 0)])
def test_config1_reads_vs_oracle(cuda_ready, kind, canonical, K, max_table, path, fs):
    """10,000 reads of 150 bp from a 100 kb genome, 1% substitutions."""
    gen = synth.genome(100_000, 1)
    rows = synth.sample_reads(gen, 10_000, 150, 0.01, 2)
    pr = synth.rows_to_packed(rows)
    sizes = oracle.primes(4, max_table)
    st, n_new_ref = _oracle_run(kind, canonical, K, sizes, pr)
    g = graph_for(kind, canonical, K, sizes)
    g.set_insert_schedule(65536, 4)
    g.set_insert_path(path)
    if fs:
        g.set_bucket_bits(fs)
    n_new = g.insert_packed(pr)
    assert np.array_equal(n_new, n_new_ref)
    check_tables(g, st.tables())
    assert (g.n_unique(), g.n_occupied()) == st.stats()
    assert np.array_equal(g.query_packed(pr), st.query_reads(canonical, K, pr.packed, pr.offsets))
    assert np.array_equal(g.neighbor_masks_packed(pr),
                          st.decision_masks(canonical, K, pr.packed, pr.offsets))


def test_batches_in_sequence_vs_oracle(cuda_ready):
    """Several batches into one graph equal one sequential pass, switching
    between the two insert paths (they share the claims map epochs)."""
    gen = synth.genome(30_000, 7)
    sizes = oracle.primes(4, 30011)
    st = oracle.Storage("byte", sizes)
    g = graph_for("byte", True, 31, sizes)
    g.set_insert_schedule(2048, 4)
    g.set_bucket_bits(6)
    for b in range(8):
        g.set_insert_path(["persistent", "windowed", "bucketed", "bucketed_ordered"][b % 4])
        rows = synth.sample_reads(gen, 700, 150, 0.02, 100 + b)
        pr = synth.rows_to_packed(rows)
        _, ref = st.insert_reads(True, 31, pr.packed, pr.offsets)
        assert np.array_equal(g.insert_packed(pr), ref)
    check_tables(g, st.tables())
    assert (g.n_unique(), g.n_occupied()) == st.stats()


def test_uneven_reads_vs_oracle(cuda_ready):
    """Log-normal lengths with indels, many zero-k-mer reads mixed in."""
    gens = [synth.genome(20_000, 50 + i) for i in range(3)]
    rs = synth.uneven_reads(gens, [1, 2, 4], 300, 400, 1.0, 5, 3000, 0.04, 0.02, 0.02, 9)
    pr = synth.list_to_packed(rs)
    sizes = oracle.primes(4, 60013)
    st, ref = _oracle_run("nibble", False, 21, sizes, pr)
    for path in ("persistent", "bucketed", "bucketed_ordered"):
        g = graph_for("nibble", False, 21, sizes)
        g.set_insert_schedule(4096, 8)
        g.set_insert_path(path)
        g.set_bucket_bits(9)
        assert np.array_equal(g.insert_packed(pr), ref)
        check_tables(g, st.tables())
        assert (g.n_unique(), g.n_occupied()) == st.stats()


def test_hash_array_insert_query_vs_oracle(cuda_ready):
    """Raw hash values, with fastmod edge values and duplicates."""
    rng = np.random.default_rng(21)
    sizes = [1000003, 999983, 65537, 3]
    edge = []
    for p in sizes:
        edge += [0, p - 1, p, p + 1, 2 * p - 1, (2**64 - 1) // p * p, 2**64 - 1]
    h = np.concatenate([np.array(edge, np.uint64), rng.integers(0, 2**64 - 1, 20000, np.uint64,
                                                                endpoint=True)])
    h = np.concatenate([h, h[:500], rng.choice(h, 3000)])
    for kind in ("bit", "byte", "nibble"):
        st = oracle.Storage(kind, sizes)
        ref_new = np.array([st.insert(int(x)) for x in h])
        g = graph_for(kind, True, 31, sizes)
        assert np.array_equal(g.insert_hashes(h), ref_new)
        check_tables(g, st.tables())
        assert (g.n_unique(), g.n_occupied()) == st.stats()
        assert np.array_equal(g.query_hashes(h), np.array([st.query(int(x)) for x in h], np.int16))


def test_mirror_semantics(cuda_ready):
    """Presence / counting semantics of the reference's tests/test_dbg.py:19-102."""
    rng = np.random.default_rng(8)
    seq = "".join(rng.choice(list("ACGT"), 60))
    for kind in ("bit", "byte", "nibble"):
        g = graph_for(kind, True, 21, oracle.primes(4, 10007))
        for i in range(len(seq) - 20):
            kmer = seq[i:i + 21]
            h = g.hash(kmer)
            assert g.query(kmer) == 0 and g.query(h) == 0
            assert g.insert(kmer) is True
            assert g.query(kmer) == 1
            assert g.insert(kmer) is False
            assert g.query(h) == (1 if kind == "bit" else 2)
        with pytest.raises(G.SequenceLengthException):
            g.insert_sequence("ATGCA")
        with pytest.raises(G.InvalidSequenceException):
            g.insert_sequence("ACGTN" * 10)
        c = g.clone()
        assert c.n_unique() == 0 and g.n_unique() > 0
        assert all(int(t.sum()) == 0 for t in c.get_raw())


def test_device_pointer_api(cuda_ready):
    import torch
    gen = synth.genome(20_000, 3)
    rows = synth.sample_reads(gen, 2000, 150, 0.01, 4)
    pr = synth.rows_to_packed(rows)
    sizes = oracle.primes(4, 20011)
    st, ref = _oracle_run("bit", True, 31, sizes, pr)
    g = graph_for("bit", True, 31, sizes)
    d_packed = torch.from_numpy(pr.packed.view(np.int32)).cuda()
    d_off = torch.from_numpy(pr.offsets.view(np.int64)).cuda()
    d_new = torch.zeros(pr.n_reads, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    g.insert_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), pr.n_reads,
                    n_new_ptr=d_new.data_ptr(), stream=s.cuda_stream)
    s.synchronize()
    assert np.array_equal(d_new.cpu().numpy().view(np.uint64), ref)
    check_tables(g, st.tables())
    nk = pr.n_kmers(31)
    d_cnt = torch.zeros(nk, dtype=torch.int16, device="cuda")
    g.query_device(d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(), pr.n_reads,
                   d_cnt.data_ptr(), n_kmers=nk, stream=s.cuda_stream)
    s.synchronize()
    assert np.array_equal(d_cnt.cpu().numpy(), st.query_reads(True, 31, pr.packed, pr.offsets))


@pytest.mark.parametrize("path", ["bucketed", "bucketed_ordered", "persistent", "windowed"])
def test_device_batch_ending_on_a_word_boundary(cuda_ready, path):
    """A device batch whose packed stream has no slack word: its bases end
    exactly at a 16-base word boundary and its last reads are exactly K long
    (their k-mer is the last one of the stream); results equal the oracle's."""
    import torch
    K = 31
    gen = synth.genome(100_000, 21)
    rows = list(synth.sample_reads(gen, 600, 90, 0.01, 22))
    rows += [rows[0][:K].copy(), rows[1][:K].copy()]
    pad = (-sum(len(r) for r in rows)) % 16
    rows[-3] = np.concatenate([rows[-3], rows[-3][:pad]])   # the stream ends on a word boundary
    pr = G.from_codes(rows)
    assert int(pr.offsets[-1]) % 16 == 0
    words = int(pr.offsets[-1]) // 16
    sizes = oracle.primes(4, 200_003)
    g = graph_for("byte", True, K, sizes)
    g.set_insert_path(path)
    d_packed = torch.from_numpy(pr.packed[:words].view(np.int32).copy()).cuda()
    d_off = torch.from_numpy(pr.offsets.view(np.int64)).cuda()
    d_new = torch.zeros(pr.n_reads, dtype=torch.int64, device="cuda")
    g.insert_device(d_packed.data_ptr(), words, d_off.data_ptr(), pr.n_reads,
                    n_new_ptr=d_new.data_ptr())
    g.synchronize()
    ref = oracle.Storage("byte", sizes)
    _, want = ref.insert_reads(True, K, pr.packed, pr.offsets)
    assert np.array_equal(d_new.cpu().numpy().view(np.uint64), want)
    for a, t in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, t)


def test_device_offsets_validated(cuda_ready):
    """Offsets that decrease or run past the packed stream are rejected on
    the device (counted as zero k-mers) and reported, without reading past
    the buffers."""
    import torch
    g = graph_for("bit", True, 31, oracle.primes(4, 10007))
    packed = torch.zeros(64, dtype=torch.int32, device="cuda")
    off = torch.tensor([0, 200, 100, 5000], dtype=torch.int64, device="cuda")
    g.insert_device(packed.data_ptr(), packed.numel(), off.data_ptr(), 3)
    with pytest.raises(G.GoetiaError):
        g.synchronize()
    assert g.device_status() == 0
    # the graph is still usable
    assert g.insert_sequence("ACGT" * 10) == 10


@pytest.mark.parametrize("path", ["bucketed", "windowed"])
def test_async_host_batches_in_flight(cuda_ready, path):
    """Large host batches through gdbg_insert_batch_async, queued back to back:
    their copies go to two staging slots in turn on the handle's second stream
    (the third call refills the first slot, regrown for a larger batch, while
    the second batch may still run; the second call counts its k-mers from the
    host offsets).  Per-read new counts, tables and counters equal those of the
    same batches through the synchronous host call."""
    import torch
    K = 31
    gen = synth.genome(2_000_000, 31)
    sizes = oracle.primes(4, 1 << 26)
    g = graph_for("byte", True, K, sizes)
    twin = graph_for("byte", True, K, sizes)
    g.set_insert_path(path)
    twin.set_insert_path(path)
    batches, held = [], []
    for b, n in enumerate((115_000, 120_000, 150_000)):
        pr = synth.rows_to_packed(synth.sample_reads(gen, n, 150, 0.005, 40 + b))
        assert pr.packed.size >= 1 << 20   # the two-slot path
        hp = torch.from_numpy(pr.packed.view(np.int32)).pin_memory()
        ho = torch.from_numpy(pr.offsets.view(np.int64)).pin_memory()
        hn = torch.zeros(max(pr.n_reads, 1), dtype=torch.int64).pin_memory()
        nk = None if b == 1 else pr.n_kmers(K)   # None: the call counts them itself
        g.insert_async(hp.data_ptr(), pr.packed.size, ho.data_ptr(), pr.n_reads, nk, hn.data_ptr())
        batches.append(pr)
        held.append((hp, ho, hn))
    g.synchronize()
    for pr, (_, _, hn) in zip(batches, held):
        want = twin.insert_packed(pr)
        assert np.array_equal(hn.numpy()[:pr.n_reads].view(np.uint64), want)
    for a, t in zip(g.get_raw(), twin.get_raw()):
        assert np.array_equal(a, t)
    assert (g.n_unique(), g.n_occupied()) == (twin.n_unique(), twin.n_occupied())


@pytest.mark.parametrize("path", ["bucketed", "windowed"])
def test_host_offsets_rejected_before_tables_change(cuda_ready, path):
    """A host batch whose offsets decrease or run past the packed stream is
    refused with INVALID_ARG by the device's offset check, before any table
    changes; a valid batch on the same handle then inserts as usual."""
    g = graph_for("byte", True, 21, oracle.primes(4, 100003))
    g.set_insert_path(path)
    rows = synth.sample_reads(synth.genome(20_000, 3), 200, 100, 0.01, 4)
    pr = synth.rows_to_packed(rows)
    g.insert_packed(pr)
    before = [t.copy() for t in g.get_raw()]
    stats = (g.n_unique(), g.n_occupied())
    bad = [pr.offsets.copy(), pr.offsets.copy()]
    bad[0][50], bad[0][51] = bad[0][51], bad[0][50]        # decreasing pair
    bad[1][-1] = pr.packed.size * 16 + 1                     # past the stream
    for off in bad:
        with pytest.raises(G.GoetiaError) as e:
            g.insert_packed(G.PackedReads(pr.packed, off))
        assert e.value.code == G._lib.ERR_INVALID_ARG
        for a, t in zip(g.get_raw(), before):
            assert np.array_equal(a, t)
        assert (g.n_unique(), g.n_occupied()) == stats
    assert g.device_status() == 0
    ref = oracle.Storage("byte", oracle.primes(4, 100003))
    ref.insert_reads(True, 21, pr.packed, pr.offsets)
    pr2 = synth.rows_to_packed(synth.sample_reads(synth.genome(20_000, 3), 100, 90, 0.01, 5))
    _, want = ref.insert_reads(True, 21, pr2.packed, pr2.offsets)
    assert np.array_equal(g.insert_packed(pr2), want)


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
def test_segmented_dense_buckets(cuda_ready, kind):
    """Tables of one or two buckets each receiving far more distinct zero
    cells than the apply's fresh-cell map holds, so every bucket is applied
    in narrower cell ranges; then a second batch on the filled tables."""
    sizes = {"bit": [250007, 249989], "byte": [30011, 29989, 29983], "nibble": [60013, 59999]}[kind]
    g = graph_for(kind, True, 25, sizes)
    g.set_insert_path("bucketed")
    gen = synth.genome(400_000, 31)
    ref = oracle.Storage(kind, sizes)
    for b in range(2):
        rows = synth.sample_reads(gen, 3000, 120, 0.01, 40 + b)
        pr = synth.rows_to_packed(rows)
        n_new = g.insert_packed(pr)
        _, want = ref.insert_reads(True, 25, pr.packed, pr.offsets)
        assert np.array_equal(n_new, want), b
    for a, t in zip(g.get_raw(), ref.tables()):
        assert np.array_equal(a, t)
    assert (g.n_unique(), g.n_occupied()) == ref.stats()


@pytest.mark.parametrize("name", names())
def test_compactor_query_golden(cuda_ready, name):
    """Second half of the reads against a graph of the first half: new / seen
    flags and masks with the read's new k-mers equal the reference's
    (find_new_segments' loop and filter_nodes with extras)."""
    c = Case(name)
    half = len(c.reads) // 2
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    for s in c.reads[:half]:
        if len(s) >= c.K:
            g.insert_sequence(s)
    flags, masks = g.compactor_query_packed(G.pack_reads(c.reads[half:]))
    assert np.array_equal(flags, c.compactor_flags)
    assert np.array_equal(masks, c.compactor_masks)
    # per sequence
    k = 0
    for s in c.reads[half:]:
        if len(s) < c.K:
            continue
        n = len(s) - c.K + 1
        new, seen, m = g.compactor_query(s)
        assert np.array_equal(new, (c.compactor_flags[k:k + n] & 1) == 1)
        assert np.array_equal(seen, (c.compactor_flags[k:k + n] & 2) == 2)
        assert np.array_equal(m, c.compactor_masks[k:k + n])
        k += n


def test_compactor_query_vs_oracle(cuda_ready):
    """Uneven reads with repeats inside reads, against a partly filled graph."""
    gens = [synth.genome(30_000, 60 + i) for i in range(3)]
    rs = synth.uneven_reads(gens, [1, 2, 4], 400, 300, 1.0, 10, 4000, 0.03, 0.01, 0.01, 19)
    rs += [np.tile(np.array([0, 1, 2, 3, 3, 1], np.uint8), 80)] * 3
    pr = synth.list_to_packed(rs)
    sizes = oracle.primes(4, 200_003)
    st = oracle.Storage("byte", sizes)
    g = graph_for("byte", True, 25, sizes)
    first = synth.list_to_packed(rs[:150])
    st.insert_reads(True, 25, first.packed, first.offsets)
    g.insert_packed(first)
    flags, masks = g.compactor_query_packed(pr)
    want_f, want_m = st.compactor_reads(True, 25, pr.packed, pr.offsets)
    assert np.array_equal(flags, want_f)
    assert np.array_equal(masks, want_m)


def test_pack_reads_device_matches_host_policy(cuda_ready):
    """The GPU packer keeps, drops and packs exactly like the host packer and
    the oracle's FASTX policy: lowercase, N and other symbols, short reads,
    empty reads, lengths around word boundaries."""
    import torch
    rng = np.random.default_rng(77)
    seqs = []
    for i in range(3000):
        L = int(rng.integers(0, 300))
        s = "".join(rng.choice(list("ACGTacgt"), L))
        if i % 7 == 0 and L:
            p = int(rng.integers(0, L))
            s = s[:p] + rng.choice(list("NnXx-.")) + s[p + 1:]
        seqs.append(s)
    seqs += ["A" * 16, "C" * 17, "g" * 15, "", "ACGTN", "T" * 1000]
    data = b"".join(s.encode() for s in seqs)
    so = np.zeros(len(seqs) + 1, np.uint64)
    so[1:] = np.cumsum([len(s) for s in seqs])
    for min_len in (0, 50):
        host = G.pack_reads(seqs, min_length=min_len)
        d_seqs = torch.from_numpy(np.frombuffer(data, np.uint8).copy()).cuda()
        d_so = torch.from_numpy(so.view(np.int64)).cuda()
        packed, offsets, kept, skipped = G.reads.pack_reads_device(d_seqs, d_so, min_len)
        torch.cuda.synchronize()
        assert kept == host.n_reads and skipped == host.n_skipped
        off = offsets.cpu().numpy().view(np.uint64)
        assert np.array_equal(off, host.offsets)
        nw = (int(off[-1]) + 15) // 16
        assert np.array_equal(packed.cpu().numpy().view(np.uint32)[:nw], host.packed[:nw])
        p2, o2, sk = oracle.pack_ascii(seqs, min_len)
        assert np.array_equal(o2, host.offsets) and sk == skipped


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
def test_fork_degrees(cuda_ready, kind):
    """A right fork, as in the reference's tests/test_traversal.py:123-151: a
    core path and a branch that shares its first 50 bases.  The k-mer ending
    at the divergence has out-degree 2 and in-degree 1 (left_degree /
    right_degree, and in_degree / out_degree on the cursor), and it is the
    decision k-mer find_decision_kmers reports on the core."""
    K, pivot = 21, 50
    rng = np.random.default_rng(12)
    core = "".join(rng.choice(list("ACGT"), 80))
    alt = "ACGT"[("ACGT".index(core[pivot]) + 1) % 4]
    branch = core[:pivot] + alt + "".join(rng.choice(list("ACGT"), 29))
    g = graph_for(kind, True, K, oracle.primes(4, 100_003))
    g.insert_sequence(core)
    g.insert_sequence(branch)
    fork = core[pivot - K:pivot]
    assert g.right_degree(fork) == 2
    assert g.left_degree(fork) == 1
    g.set_cursor(fork)
    assert (g.in_degree(), g.out_degree(), g.degree()) == (1, 2, 3)
    pos, hs = g.find_decision_kmers(core)
    assert pos == [pivot - K]
    assert int(hs[0]) == int(g.hash(fork))
    # a k-mer inside the core path away from the fork: one in, one out
    assert (g.left_degree(core[10:10 + K]), g.right_degree(core[10:10 + K])) == (1, 1)
