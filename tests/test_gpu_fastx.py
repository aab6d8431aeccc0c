"""The GPU FASTX parser (gdbg_parse_fastx_device) against the reference's
FastxParser<DNA_SIMPLE>.

Every case of tests/golden/fastx.npz (written by the reference's own parser,
tests/golden/make_fastx_golden.py) goes through the device parser: regular
layouts must give exactly the reads next() returned -- packed like the host
packer packs them -- and the reference's n_parsed / n_skipped; the "x_"
cases, which the parser does not take, must raise ERR_UNSUPPORTED so the
caller parses them on the host.  Larger seeded texts are compared with the
oracle's kseq restatement (itself pinned to the same fixture), from aligned
and unaligned device pointers, and a parsed FASTQ batch inserted into a dBG
gives the same per-read new counts as the host-packed reads."""
import os

import numpy as np
import pytest

import oracle
import goetia_gb300 as G
from goetia_gb300 import _lib

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def golden():
    return np.load(os.path.join(HERE, "golden", "fastx.npz"))


def device_text(text, offset=0):
    """text on the device, starting `offset` bytes into its allocation."""
    import torch
    buf = torch.zeros(len(text) + offset + 16, dtype=torch.uint8, device="cuda")
    if text:
        buf[offset:offset + len(text)] = torch.from_numpy(np.frombuffer(text, np.uint8).copy()).cuda()
    return buf[offset:offset + len(text)]


def check_against(seqs, stats_expect, packed, offsets, stats, what):
    host = G.pack_reads([s.decode() for s in seqs])
    assert host.n_skipped == 0, what   # the expected reads are all valid
    off = offsets.cpu().numpy().view(np.uint64)
    assert stats["n_kept"] == len(seqs), what
    assert np.array_equal(off, host.offsets), what
    nw = (int(off[-1]) + 15) // 16
    assert np.array_equal(packed.cpu().numpy().view(np.uint32)[:nw], host.packed[:nw]), what
    assert stats["n_parsed"] == stats_expect[0] and stats["n_skipped"] == stats_expect[1], what
    assert stats["n_dropped"] == stats["n_parsed"] - stats["n_kept"], what


@pytest.mark.parametrize("offset", [0, 3])
def test_fastx_golden_cases(cuda_ready, offset):
    z = golden()
    for name in z["names"]:
        text = z[name + "__text"].tobytes()
        d = device_text(text, offset)
        for ml in z["min_lengths"]:
            k = f"{name}__m{ml}"
            if name.startswith("x_"):
                with pytest.raises(_lib.GoetiaError) as ei:
                    G.reads.parse_fastx_device(d, int(ml))
                assert ei.value.code == _lib.ERR_UNSUPPORTED, k
                continue
            seq, off, st = z[k + "__seq"].tobytes(), z[k + "__off"], z[k + "__stats"]
            assert not st[2], k
            gold = [seq[int(off[i]):int(off[i + 1])] for i in range(len(off) - 1)]
            packed, offsets, stats = G.reads.parse_fastx_device(d, int(ml))
            check_against(gold, (int(st[0]), int(st[1])), packed, offsets, stats, k)


def _fastq(rng, n, crlf=False):
    nl = b"\r\n" if crlf else b"\n"
    out = []
    for i in range(n):
        L = int(rng.integers(0, 400))
        s = bytearray(rng.choice(list(b"ACGTacgt"), L).astype(np.uint8).tobytes())
        if i % 13 == 0 and L:
            s[int(rng.integers(0, L))] = ord(rng.choice(list("NRY.")))
        out.append(b"@r%d x\t%d" % (i, i) + nl + bytes(s) + nl + b"+" + nl + b"F" * L + nl)
    return b"".join(out)


def _fasta(rng, n, width):
    out = []
    for i in range(n):
        L = int(rng.integers(0, 3000))
        s = rng.choice(list(b"ACGTacgtN"), L, p=[.24, .24, .24, .24, .01, .01, .01, .005, .005])
        s = s.astype(np.uint8).tobytes()
        out.append((b">" if i % 5 else b"@") + b"c%d\n" % i +
                   b"".join(s[j:j + width] + b"\n" for j in range(0, len(s), width)))
    return b"".join(out)


@pytest.mark.parametrize("kind", ["fastq", "fastq_crlf", "fasta60", "fasta_one_line"])
def test_fastx_large_vs_oracle(cuda_ready, kind):
    rng = np.random.default_rng({"fastq": 1, "fastq_crlf": 2, "fasta60": 3, "fasta_one_line": 4}[kind])
    if kind.startswith("fastq"):
        text = _fastq(rng, 20000, crlf=kind.endswith("crlf"))
    else:
        text = _fasta(rng, 3000, 60 if kind == "fasta60" else 1 << 20)
    for offset in (0, 1):
        d = device_text(text, offset)
        for ml in (0, 100):
            seqs, st, status = oracle.parse_fastx(text, ml)
            assert status == 0
            packed, offsets, stats = G.reads.parse_fastx_device(d, ml)
            check_against(seqs, (st["n_parsed"], st["n_skipped"]), packed, offsets, stats,
                          f"{kind} offset {offset} min_length {ml}")


def test_fastx_offsets_capacity(cuda_ready):
    """Too few offsets entries: GDBG_ERR_INVALID_ARG with the record count set."""
    import ctypes
    import torch
    text = b"@a\nACGT\n+\nIIII\n@b\nGG\n+\nII\n@c\nT\n+\nI\n"
    d = device_text(text)
    packed = torch.zeros(8, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(2, dtype=torch.int64, device="cuda")
    st = np.zeros(4, np.uint64)
    rc = _lib.load().gdbg_parse_fastx_device(
        ctypes.c_void_p(d.data_ptr()), len(text), 0, ctypes.c_void_p(packed.data_ptr()), 8,
        ctypes.c_void_p(offsets.data_ptr()), 2, st.ctypes.data_as(_lib.u64p), None)
    assert rc == _lib.ERR_INVALID_ARG and int(st[2]) == 3


def test_fastx_batch_inserts_like_host_packed(cuda_ready):
    """A FASTQ batch parsed on the GPU and inserted gives the per-read new
    counts and tables of the same reads packed on the host."""
    import torch
    rng = np.random.default_rng(8)
    g0 = rng.integers(0, 4, 20000, dtype=np.uint8)
    reads = []
    for i in range(3000):
        s = int(rng.integers(0, len(g0) - 150))
        r = "".join("ACGT"[c] for c in g0[s:s + 150])
        if i % 50 == 0:
            r = r[:70] + "N" + r[71:]
        reads.append(r)
    text = b"".join(b"@q%d\n%s\n+\n%s\n" % (i, r.encode(), b"I" * len(r)) for i, r in enumerate(reads))
    packed, offsets, stats = G.reads.parse_fastx_device(device_text(text))
    host = G.pack_reads(reads)
    assert stats["n_kept"] == host.n_reads and stats["n_skipped"] == host.n_skipped
    sizes = oracle.primes(4, 200_003)
    Graph = G.dBG[G.ByteStorage, G.CanLemireShifter]
    a = Graph.build(G.ByteStorage(tablesizes=sizes), 31)
    b = Graph.build(G.ByteStorage(tablesizes=sizes), 31)
    n_kept = stats["n_kept"]
    d_new = torch.zeros(n_kept, dtype=torch.int64, device="cuda")
    a.insert_device(packed.data_ptr(), packed.numel(), offsets.data_ptr(), n_kept,
                    n_new_ptr=d_new.data_ptr())
    a.synchronize()
    n_new_host = b.insert_packed(host)
    assert np.array_equal(d_new.cpu().numpy(), np.asarray(n_new_host, np.int64))
    for ta, tb in zip(a.get_raw(), b.get_raw()):
        assert np.array_equal(ta, tb)


def test_fastx_kernel_follows_the_per_line_rule(cuda_ready):
    """Seeded random FASTA / FASTQ-like texts (the line kinds of
    tests/test_fastx_rule.py): the GPU parser declines exactly the texts the
    per-line rule declines, and elsewhere gives kseq's reads and counts."""
    import test_fastx_rule as rule
    rng = np.random.default_rng(5)
    seen = {True: 0, False: 0}
    for _ in range(800):
        text = rule.random_text(rng)
        d = device_text(text, int(rng.integers(0, 4)))
        for ml in (0, 4):
            expect = rule.per_line_rule(text, ml)
            seen[expect is None] += 1
            if expect is None:
                with pytest.raises(_lib.GoetiaError) as ei:
                    G.reads.parse_fastx_device(d, ml)
                assert ei.value.code == _lib.ERR_UNSUPPORTED, text
                continue
            seqs, st, status = oracle.parse_fastx(text, ml)
            assert status == 0 and (seqs, st["n_parsed"], st["n_skipped"]) == expect, text
            packed, offsets, stats = G.reads.parse_fastx_device(d, ml)
            check_against(seqs, (st["n_parsed"], st["n_skipped"]), packed, offsets, stats, text)
    assert seen[True] > 80 and seen[False] > 80
