"""The CPU oracle (oracle/goetia_oracle.c) pinned against the reference.

Pins: the K=27 known-answer hash from the reference's own tests
(tests/test_hashing.py:15-19) and the golden fixtures written by the
reference's C++ objects (tests/golden/make_golden.py).  CPU only.
"""
import numpy as np
import pytest

import oracle
from goldens import Case, names

KNOWN_KMER = "TCACCTGTGTTGTGCTACTTGCGGCGC"
KNOWN_FWD = 13194817695400542713
KNOWN_RC = 4324216031038051805


def codes(s):
    return np.array(["ACGT".index(c) for c in s], np.uint8)


def test_known_answer_k27():
    fw, rc = oracle.hash_codes(codes(KNOWN_KMER), 27)
    assert int(fw[0]) == KNOWN_FWD
    assert int(rc[0]) == KNOWN_RC
    assert min(int(fw[0]), int(rc[0])) == KNOWN_RC   # known_can = known_rc


def test_rolling_equals_recomputed():
    rng = np.random.default_rng(5)
    s = rng.integers(0, 4, 300, dtype=np.uint8)
    for K in (1, 21, 31, 63, 64, 65, 101, 128):
        fw, rc = oracle.hash_codes(s, K)
        for p in (0, 1, 17, len(s) - K):
            f1, r1 = oracle.hash_codes(s[p:p + K], K)
            assert fw[p] == f1[0] and rc[p] == r1[0]
            # canonical == min(fw(kmer), fw(revcomp(kmer))) (test_hashing.py:161-172)
            frc, _ = oracle.hash_codes((3 - s[p:p + K][::-1]).astype(np.uint8), K)
            assert rc[p] == frc[0]


def test_primes():
    # config 1 table sizes, verified against get_n_primes_near_x
    assert oracle.primes(4, 4194304) == [4194301, 4194287, 4194277, 4194271]
    assert oracle.primes(3, 10) == [7, 5, 3]
    assert oracle.primes(1, 1) == [1]


@pytest.mark.parametrize("name", names())
def test_oracle_matches_golden(name):
    c = Case(name)
    packed, off = c.packed()
    val, fw, rc = oracle.hash_reads(c.canonical, c.K, packed, off)
    assert np.array_equal(val, c.val)
    if c.canonical:
        assert np.array_equal(fw, c.fw) and np.array_equal(rc, c.rc)
    st = oracle.Storage(c.storage, c.sizes)
    total, n_new = st.insert_reads(c.canonical, c.K, packed, off)
    assert total == int(c.n_kmers.sum())
    assert np.array_equal(n_new, c.n_new)
    for a, b in zip(st.tables(), c.tables):
        assert np.array_equal(a, b)
    assert st.stats() == (c.n_unique, c.n_occupied)
    assert np.array_equal(st.query_reads(c.canonical, c.K, packed, off), c.counts)
    masks = st.decision_masks(c.canonical, c.K, packed, off)
    assert np.array_equal(masks, c.masks)
    assert c.decision_positions(masks) == c.dpos
    # insert_and_query_sequence per read on fresh tables
    st2 = oracle.Storage(c.storage, c.sizes)
    assert np.array_equal(st2.insert_and_query_reads(c.canonical, c.K, packed, off), c.iq_counts)
    # the OXLI file written by the reference's dBG::save, byte for byte
    u, o = st.stats()
    assert oracle.oxli_bytes(c.storage, c.K, c.sizes, st.tables(), o) == c.oxli
    kind, K, sizes, tables, occ = oracle.parse_oxli(c.oxli)
    assert (K, occ, sizes) == (c.K, c.n_occupied, [int(x) for x in c.sizes])
    assert all(np.array_equal(a, b) for a, b in zip(tables, c.tables))


@pytest.mark.parametrize("name", [n for n in names() if n.startswith("bit")])
def test_oracle_update_from_matches_golden(name):
    c = Case(name)
    half = len(c.reads) // 2
    sa, sb = oracle.Storage("bit", c.sizes), oracle.Storage("bit", c.sizes)
    for st, part in ((sa, c.reads[:half]), (sb, c.reads[half:])):
        packed, off, _ = oracle.pack_ascii(part)
        st.insert_reads(c.canonical, c.K, packed, off)
    (ua, oa), (ub, ob) = sa.stats(), sb.stats()
    assert [ua, oa, ub, ob] == [int(x) for x in c.merge_stats[:4]]
    merged, occ = oracle.update_from(sa.tables(), sb.tables(), oa)
    assert occ == int(c.merge_stats[5]) and ua == int(c.merge_stats[4])
    assert all(np.array_equal(a, b) for a, b in zip(merged, c.merged))


@pytest.mark.parametrize("name", names())
def test_oracle_compactor_matches_golden(name):
    c = Case(name)
    half = len(c.reads) // 2
    st = oracle.Storage(c.storage, c.sizes)
    packed, off, _ = oracle.pack_ascii(c.reads[:half])
    st.insert_reads(c.canonical, c.K, packed, off)
    packed, off, _ = oracle.pack_ascii(c.reads[half:])
    flags, masks = st.compactor_reads(c.canonical, c.K, packed, off)
    assert np.array_equal(flags, c.compactor_flags)
    assert np.array_equal(masks, c.compactor_masks)


def test_pack_policy():
    reads = ["ACGT", "acgtN", "aCgT", "", "ACGX", "TTTT"]
    packed, off, skipped = oracle.pack_ascii(reads)
    assert skipped == 2
    assert list(off) == [0, 4, 8, 8, 12]
    assert packed[0] & 0xFF == 0b11100100  # A C G T -> 0 1 2 3


def _packed_reads(rng, genome_len, n_reads, read_len):
    genome = rng.integers(0, 4, genome_len, dtype=np.uint8)
    starts = rng.integers(0, genome_len - read_len, n_reads)
    codes = np.concatenate([genome[s:s + read_len] for s in starts]).astype(np.uint32)
    idx = np.arange(len(codes), dtype=np.uint64)
    packed = np.zeros(len(codes) // 16 + 1, np.uint32)
    np.bitwise_or.at(packed, idx >> 4, codes << (2 * (idx & 15)).astype(np.uint32))
    offsets = np.arange(0, len(codes) + 1, read_len, dtype=np.uint64)
    return packed, offsets


@pytest.mark.parametrize("kind", ["bit", "byte", "nibble"])
def test_multithreaded_insert_equals_sequential(kind):
    """The reference arm's insert on several threads over one shared storage:
    cell updates are atomic and saturating increments commute, so the tables
    equal one sequential pass over the same reads.  Small tables saturate
    many Byte and Nibble cells while the threads race on them."""
    packed, offsets = _packed_reads(np.random.default_rng(7), 20_000, 3000, 150)
    sizes = oracle.primes(4, 2003)
    seq = oracle.Storage(kind, sizes)
    total, _ = seq.insert_reads(True, 31, packed, offsets)
    par = oracle.Storage(kind, sizes)
    assert par.insert_reads_mt(True, 31, packed, offsets, 4) == total == 3000 * 120
    for a, b in zip(seq.tables(), par.tables()):
        assert np.array_equal(a, b)
    if kind == "byte":
        assert any((t == 255).any() for t in seq.tables())          # saturated cells
    elif kind == "nibble":
        assert any(((t >> 4) == 15).any() for t in seq.tables())


def _fastx_golden():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "fastx.npz"))


def test_fastx_parser_vs_reference():
    """The oracle's kseq / FastxParser restatement against what the
    reference's own FastxParser<DNA_SIMPLE> returned for every FASTX case
    (tests/golden/make_fastx_golden.py): kept sequences, n_parsed,
    n_skipped (double counts included) and the InvalidRead throw."""
    z = _fastx_golden()
    for name in z["names"]:
        text = z[name + "__text"].tobytes()
        for ml in z["min_lengths"]:
            k = f"{name}__m{ml}"
            seq, off, st = z[k + "__seq"].tobytes(), z[k + "__off"], z[k + "__stats"]
            gold = [seq[int(off[i]):int(off[i + 1])] for i in range(len(off) - 1)]
            got, stats, status = oracle.parse_fastx(text, int(ml))
            assert got == gold, k
            assert (stats["n_parsed"], stats["n_skipped"]) == (int(st[0]), int(st[1])), k
            assert (status == -2) == bool(st[2]), k
