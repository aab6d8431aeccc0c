"""Whole-table operations through the C ABI: OXLI v4 files (gdbg_save /
gdbg_load) and the Bit OR-merge (gdbg_update_from).

The files the GPU library writes are compared byte for byte with the ones the
reference's dBG::save wrote for the same reads (tests/golden/*.npz "oxli"),
and the reference's files are loaded back onto the device: tables, sizes,
n_occupied and the query answers must match.  Error behaviour follows
Storage::load (bitstorage.cc:188-307): wrong signature, version or type and
truncated files raise GoetiaFileException and leave the graph as it was."""
import gzip
import os

import numpy as np
import pytest

import oracle
from goldens import Case, names
import goetia_gb300 as G
from goetia_gb300 import synth
from goetia_gb300.reads import PackedReads, codes_to_str

pytestmark = pytest.mark.gpu

STORAGES = {"bit": G.BitStorage, "byte": G.ByteStorage, "nibble": G.NibbleStorage}
SHIFTERS = {True: G.CanLemireShifter, False: G.FwdLemireShifter}


def graph_for(kind, canonical, K, sizes):
    st = STORAGES[kind](tablesizes=[int(s) for s in sizes])
    return G.dBG[STORAGES[kind], SHIFTERS[canonical]].build(st, K)


def filled(c):
    g = graph_for(c.storage, c.canonical, c.K, c.sizes)
    packed, off = c.packed()
    g.insert_packed(PackedReads(packed, off))
    return g


@pytest.mark.parametrize("name", names())
def test_save_matches_reference_file(cuda_ready, tmp_path, name):
    c = Case(name)
    g = filled(c)
    f = tmp_path / "g.oxli"
    g.save(str(f))
    assert f.read_bytes() == c.oxli


@pytest.mark.parametrize("name", names())
def test_load_reference_file(cuda_ready, tmp_path, name):
    """Load into a graph with other table sizes and a different n_occupied:
    the file's sizes, tables and occupied count replace them; K is kept."""
    c = Case(name)
    f = tmp_path / "ref.oxli"
    f.write_bytes(c.oxli)
    g = graph_for(c.storage, c.canonical, c.K, [1009, 1013])
    g.insert_sequence("ACGT" * 40)
    n_unique = g.n_unique()
    ks = g.load(str(f))
    assert ks == c.K and g.K == c.K
    assert g.storage.get_tablesizes() == [int(x) for x in c.sizes]
    for a, b in zip(g.get_raw(), c.tables):
        assert np.array_equal(a, b)
    assert g.n_occupied() == c.n_occupied
    assert g.n_unique() == n_unique            # not part of the file
    k = 0
    for s in c.reads:
        if len(s) < c.K:
            continue
        n = len(s) - c.K + 1
        assert g.query_sequence(s) == [int(x) for x in c.counts[k:k + n]]
        k += n
    # and it keeps inserting like the reference graph it came from
    g2 = filled(c)
    probe = codes_to_str(synth.genome(400, 99))
    assert g.insert_sequence_new(probe) == g2.insert_sequence_new(probe)
    for a, b in zip(g.get_raw(), g2.get_raw()):
        assert np.array_equal(a, b)


def test_byte_gz_round_trip(cuda_ready, tmp_path):
    c = Case("byte_can_k31")
    g = filled(c)
    f = tmp_path / "g.oxli.gz"
    g.save(str(f))
    assert gzip.decompress(f.read_bytes()) == c.oxli
    h = graph_for(c.storage, c.canonical, c.K, c.sizes)
    h.load(str(f))
    for a, b in zip(h.get_raw(), c.tables):
        assert np.array_equal(a, b)


def test_bit_gz_name_is_plain(cuda_ready, tmp_path):
    """BitStorage::save ignores the suffix (bitstorage.cc:151-186)."""
    c = Case("bit_can_k31")
    g = filled(c)
    f = tmp_path / "g.oxli.gz"
    g.save(str(f))
    assert f.read_bytes() == c.oxli


def test_load_errors_leave_graph_unchanged(cuda_ready, tmp_path):
    c = Case("bit_can_k31")
    g = filled(c)
    before = g.get_raw()
    occ = g.n_occupied()
    cases = {
        "sig": b"OXLX" + c.oxli[4:],
        "version": c.oxli[:4] + bytes([3]) + c.oxli[5:],
        "type": c.oxli[:5] + bytes([1]) + c.oxli[6:],
        "truncated": c.oxli[:-10],
        "header_only": c.oxli[:9],
    }
    msgs = {"sig": "signature", "version": "version", "type": "type",
            "truncated": "Unexpected end", "header_only": "Unexpected end"}
    for k, data in cases.items():
        f = tmp_path / f"{k}.oxli"
        f.write_bytes(data)
        with pytest.raises(G.GoetiaFileException, match=msgs[k]):
            g.load(str(f))
        for a, b in zip(g.get_raw(), before):
            assert np.array_equal(a, b)
        assert g.n_occupied() == occ
    with pytest.raises(G.GoetiaFileException, match="Cannot open"):
        g.load(str(tmp_path / "missing.oxli"))
    # a Byte file is the wrong type for a Bit graph
    f = tmp_path / "byte.oxli"
    f.write_bytes(Case("byte_can_k31").oxli)
    with pytest.raises(G.GoetiaFileException, match="type"):
        g.load(str(f))


def test_bigcount_file_unsupported(cuda_ready, tmp_path):
    c = Case("byte_can_k31")
    data = bytearray(c.oxli)
    data[6] = 1                      # use_bigcount
    f = tmp_path / "big.oxli"
    f.write_bytes(bytes(data))
    g = filled(c)
    with pytest.raises(G.GoetiaError, match="bigcount"):
        g.load(str(f))


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
def test_large_round_trip(cuda_ready, tmp_path, kind):
    """Tables of ~2^27 cells (files of 16-128 MB, several staging chunks):
    save, load into a fresh graph of another shape, compare against the
    oracle's file for the same tables."""
    sizes = oracle.primes(3, 1 << 27)
    g = graph_for(kind, True, 31, sizes)
    rows = synth.sample_reads(synth.genome(2_000_000, 3), 200_000, 150, 0.01, 4)
    g.insert_packed(synth.rows_to_packed(rows))
    f = tmp_path / "big.oxli"
    g.save(str(f))
    tables = g.get_raw()
    want = oracle.oxli_bytes(kind, 31, sizes, tables, g.n_occupied())
    assert os.path.getsize(f) == len(want)
    assert f.read_bytes() == want
    h = graph_for(kind, True, 31, [101])
    h.load(str(f))
    assert h.storage.get_tablesizes() == sizes
    for a, b in zip(h.get_raw(), tables):
        assert np.array_equal(a, b)
    assert h.n_occupied() == g.n_occupied()


@pytest.mark.parametrize("name", [n for n in names() if n.startswith("bit")])
def test_update_from_matches_reference(cuda_ready, name):
    """A (first half of the reads) .update_from(B) (second half): tables and
    counters equal the reference's (bitstorage.cc:103-137)."""
    c = Case(name)
    half = len(c.reads) // 2
    ga = graph_for("bit", c.canonical, c.K, c.sizes)
    gb = graph_for("bit", c.canonical, c.K, c.sizes)
    for g, part in ((ga, c.reads[:half]), (gb, c.reads[half:])):
        g.insert_packed(G.pack_reads(part))
    assert [ga.n_unique(), ga.n_occupied(), gb.n_unique(), gb.n_occupied()] == \
        [int(x) for x in c.merge_stats[:4]]
    ga.update_from(gb)
    assert (ga.n_unique(), ga.n_occupied()) == (int(c.merge_stats[4]), int(c.merge_stats[5]))
    for a, b in zip(ga.get_raw(), c.merged):
        assert np.array_equal(a, b)
    # B is unchanged; merging again adds nothing
    ga.update_from(gb)
    assert ga.n_occupied() == int(c.merge_stats[5])


def test_update_from_errors(cuda_ready):
    a = graph_for("bit", True, 31, [1009, 1013])
    with pytest.raises(G.GoetiaError, match="same table sizes"):
        a.update_from(graph_for("bit", True, 31, [1009, 1019]))
    with pytest.raises(G.GoetiaError, match="BitStorage only"):
        graph_for("byte", True, 31, [1009, 1013]).update_from(graph_for("byte", True, 31, [1009, 1013]))


def test_update_from_large(cuda_ready):
    """~2^27-cell tables: the merge against the oracle's byte-wise OR."""
    sizes = oracle.primes(4, 1 << 27)
    g1 = graph_for("bit", True, 31, sizes)
    g2 = graph_for("bit", True, 31, sizes)
    gen = synth.genome(3_000_000, 8)
    g1.insert_packed(synth.rows_to_packed(synth.sample_reads(gen, 150_000, 150, 0.01, 9)))
    g2.insert_packed(synth.rows_to_packed(synth.sample_reads(gen, 150_000, 150, 0.01, 10)))
    ta, tb, occ = g1.get_raw(), g2.get_raw(), g1.n_occupied()
    want, want_occ = oracle.update_from(ta, tb, occ)
    g1.update_from(g2)
    assert g1.n_occupied() == want_occ
    for a, b in zip(g1.get_raw(), want):
        assert np.array_equal(a, b)


def test_graphs_on_one_storage_share_tables(cuda_ready, tmp_path):
    """dBG::build on a storage already in use shares its tables and counters
    (dbg.hh:73, 97-101); clone() gets a new, empty storage."""
    c = Case("byte_can_k31")
    st = G.ByteStorage(tablesizes=[int(x) for x in c.sizes])
    Graph = G.dBG[G.ByteStorage, G.CanLemireShifter]
    g1 = Graph.build(st, c.K)
    g2 = Graph.build(st, c.K)
    half = len(c.reads) // 2
    for s in c.reads[:half]:
        if len(s) >= c.K:
            g1.insert_sequence(s)
    for s in c.reads[half:]:
        if len(s) >= c.K:
            g2.insert_sequence(s)
    # both handles see the reference's final tables and counters
    for g in (g1, g2):
        for a, b in zip(g.get_raw(), c.tables):
            assert np.array_equal(a, b)
        assert (g.n_unique(), g.n_occupied()) == (c.n_unique, c.n_occupied)
    # a graph of another K and shifter on the same storage queries the same cells
    g3 = G.dBG[G.ByteStorage, G.FwdLemireShifter].build(st, 21)
    assert g3.storage is st
    cl = g1.clone()
    assert cl.n_unique() == 0 and all(not t.any() for t in cl.get_raw())
    # the storage keeps the tables alive after its graphs are gone
    del g1, g2, g3
    g4 = Graph.build(st, c.K)
    for a, b in zip(g4.get_raw(), c.tables):
        assert np.array_equal(a, b)
    # load through one handle: the shared storage takes the file's sizes
    g5 = Graph.build(st, c.K)
    f = tmp_path / "other.oxli"
    other = graph_for("byte", True, c.K, [1009, 1013, 1019])
    other.insert_sequence(c.reads[0])
    other.save(str(f))
    g4.load(str(f))
    assert st.get_tablesizes() == [1009, 1013, 1019]
    assert g5.query_sequence(c.reads[0]) == other.query_sequence(c.reads[0])


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
def test_storage_counters_follow_its_graphs(cuda_ready, kind):
    """Storage-level n_unique_kmers / n_occupied / estimated_fp
    (bitstorage.hh:173-187) read the tables shared by every graph built on
    the storage: zero before the first graph, then the oracle's counts after
    inserts through two graphs on it."""
    sizes = oracle.primes(4, 40009)
    st = STORAGES[kind](tablesizes=sizes)
    assert (st.n_unique_kmers(), st.n_occupied()) == (0, 0)
    a = G.dBG[STORAGES[kind], G.CanLemireShifter].build(st, 31)
    b = G.dBG[STORAGES[kind], G.CanLemireShifter].build(st, 31)
    gen = synth.genome(30_000, 5)
    first = synth.rows_to_packed(synth.sample_reads(gen, 300, 150, 0.01, 6))
    second = synth.rows_to_packed(synth.sample_reads(gen, 300, 150, 0.01, 7))
    a.insert_packed(first)
    b.insert_packed(second)
    ref = oracle.Storage(kind, sizes)
    for pr in (first, second):
        ref.insert_reads(True, 31, pr.packed, pr.offsets)
    assert (st.n_unique_kmers(), st.n_occupied()) == ref.stats()
    assert (a.n_unique(), a.n_occupied()) == (b.n_unique(), b.n_occupied()) == ref.stats()
    assert st.estimated_fp() == a.estimated_fp() > 0
