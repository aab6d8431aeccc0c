"""CPU oracle for the goetia dBG hot path -- TEST INFRASTRUCTURE ONLY.

ctypes front end over ``oracle/_build/liboracle.so``, the plain-C restatement
of the reference algorithm in ``goetia_oracle.c``.  Only the tests, the smoke
check and the benchmark's CPU-baseline leg use this module, as the checker;
the product path (``goetia_gb300``) never imports it.

Read batches use the same encoding as the GPU library: a packed 2-bit base
stream (``uint32``, 16 bases per word) plus ``n_reads + 1`` base offsets.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

BIT, BYTE, NIBBLE = 0, 1, 2
KINDS = {"bit": BIT, "byte": BYTE, "nibble": NIBBLE}

_lib = None

u64p = ctypes.POINTER(ctypes.c_uint64)
u32p = ctypes.POINTER(ctypes.c_uint32)
u8p = ctypes.POINTER(ctypes.c_uint8)
i16p = ctypes.POINTER(ctypes.c_int16)


def build():
    """Compile the C restatement (gcc, a second or two)."""
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    src = os.path.join(HERE, "goetia_oracle.c")
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-pthread",
                           "-o", tmp, src])
    os.replace(tmp, LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "goetia_oracle.c")
        if (not os.path.exists(LIB_PATH)
                or os.path.getmtime(LIB_PATH) < os.path.getmtime(src)):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_storage_new.restype = ctypes.c_void_p
        L.orc_storage_new.argtypes = [ctypes.c_int, u64p, ctypes.c_int]
        L.orc_storage_free.argtypes = [ctypes.c_void_p]
        L.orc_table_bytes.restype = ctypes.c_uint64
        L.orc_table_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_table.restype = u8p
        L.orc_table.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_stats.argtypes = [ctypes.c_void_p, u64p, u64p]
        L.orc_insert.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_query.restype = ctypes.c_int16
        L.orc_query.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_insert_and_query.restype = ctypes.c_int16
        L.orc_insert_and_query.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_primes.restype = ctypes.c_uint32
        L.orc_primes.argtypes = [ctypes.c_uint32, ctypes.c_uint64, u64p]
        L.orc_hash_codes.argtypes = [u8p, ctypes.c_uint64, ctypes.c_uint16, u64p, u64p]
        L.orc_count_kmers.restype = ctypes.c_uint64
        L.orc_count_kmers.argtypes = [ctypes.c_uint16, u64p, ctypes.c_uint64]
        batch = [ctypes.c_int, ctypes.c_uint16, u32p, u64p, ctypes.c_uint64]
        L.orc_hash_reads.argtypes = batch + [u64p, u64p, u64p]
        L.orc_insert_reads.restype = ctypes.c_uint64
        L.orc_insert_reads.argtypes = [ctypes.c_void_p] + batch + [u64p]
        L.orc_insert_and_query_reads.argtypes = [ctypes.c_void_p] + batch + [i16p]
        L.orc_query_reads.argtypes = [ctypes.c_void_p] + batch + [i16p]
        L.orc_decision_masks.argtypes = [ctypes.c_void_p] + batch + [u8p]
        L.orc_compactor_reads.argtypes = [ctypes.c_void_p] + batch + [u8p, u8p]
        L.orc_insert_reads_mt.restype = ctypes.c_uint64
        L.orc_insert_reads_mt.argtypes = [ctypes.c_void_p] + batch + [ctypes.c_int]
        L.orc_pack_ascii.restype = ctypes.c_int64
        L.orc_pack_ascii.argtypes = [ctypes.c_char_p, u64p, ctypes.c_uint64, ctypes.c_uint32,
                                     u32p, u64p, u64p]
        L.orc_parse_fastx.restype = ctypes.c_int64
        L.orc_parse_fastx.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_char_p, ctypes.c_uint64, u64p, ctypes.c_uint64,
                                      u64p]
        L.orc_symbol_table.argtypes = [u64p]
        L.orc_count_cells.restype = ctypes.c_int
        L.orc_count_cells.argtypes = [ctypes.c_int, ctypes.c_uint16, u32p, u64p, ctypes.c_uint64,
                                      u64p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, u64p,
                                      ctypes.c_uint64, u8p, ctypes.c_int]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def primes(n, x):
    out = np.zeros(max(n, 1), np.uint64)
    got = lib().orc_primes(n, x, _p(out, u64p))
    return [int(v) for v in out[:got]]


def hash_codes(codes, K):
    """fw/rc rolling hashes of a code array (eat + update, cyclichash.h)."""
    codes = np.ascontiguousarray(codes, np.uint8)
    n = max(len(codes) - K + 1, 0)
    fw = np.zeros(n, np.uint64)
    rc = np.zeros(n, np.uint64)
    if n:
        lib().orc_hash_codes(_p(codes, u8p), len(codes), K, _p(fw, u64p), _p(rc, u64p))
    return fw, rc


class Storage:
    """Bit/Byte/Nibble storage with the reference's sequential semantics."""

    def __init__(self, kind, sizes):
        self.kind = KINDS[kind] if isinstance(kind, str) else kind
        self.sizes = np.ascontiguousarray(sizes, np.uint64)
        self.h = lib().orc_storage_new(self.kind, _p(self.sizes, u64p), len(self.sizes))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_storage_free(self.h)
            self.h = None

    def insert(self, h):
        return bool(lib().orc_insert(self.h, int(h)))

    def query(self, h):
        return int(lib().orc_query(self.h, int(h)))

    def insert_and_query(self, h):
        return int(lib().orc_insert_and_query(self.h, int(h)))

    def tables(self):
        L = lib()
        out = []
        for i in range(len(self.sizes)):
            n = L.orc_table_bytes(self.h, i)
            out.append(np.ctypeslib.as_array(L.orc_table(self.h, i), shape=(n,)).copy())
        return out

    def table_view(self, i):
        """Table i's bytes without a copy (valid while the storage lives)."""
        L = lib()
        n = L.orc_table_bytes(self.h, i)
        return np.ctypeslib.as_array(L.orc_table(self.h, i), shape=(n,))

    def stats(self):
        u, o = ctypes.c_uint64(), ctypes.c_uint64()
        lib().orc_stats(self.h, ctypes.byref(u), ctypes.byref(o))
        return int(u.value), int(o.value)

    # -- read batches ------------------------------------------------------
    def insert_reads(self, canonical, K, packed, offsets):
        n = len(offsets) - 1
        n_new = np.zeros(max(n, 1), np.uint64)
        total = lib().orc_insert_reads(self.h, int(canonical), K, _p(packed, u32p),
                                       _p(offsets, u64p), n, _p(n_new, u64p))
        return int(total), n_new[:n]

    def insert_reads_mt(self, canonical, K, packed, offsets, threads):
        n = len(offsets) - 1
        return int(lib().orc_insert_reads_mt(self.h, int(canonical), K, _p(packed, u32p),
                                             _p(offsets, u64p), n, threads))

    def insert_and_query_reads(self, canonical, K, packed, offsets):
        nk = count_kmers(K, offsets)
        out = np.zeros(max(nk, 1), np.int16)
        lib().orc_insert_and_query_reads(self.h, int(canonical), K, _p(packed, u32p),
                                         _p(offsets, u64p), len(offsets) - 1, _p(out, i16p))
        return out[:nk]

    def query_reads(self, canonical, K, packed, offsets):
        nk = count_kmers(K, offsets)
        out = np.zeros(max(nk, 1), np.int16)
        lib().orc_query_reads(self.h, int(canonical), K, _p(packed, u32p), _p(offsets, u64p),
                              len(offsets) - 1, _p(out, i16p))
        return out[:nk]

    def compactor_reads(self, canonical, K, packed, offsets):
        """Per k-mer (flags, masks) of the compactor query: bit 0 new, bit 1
        seen; masks over the storage plus each read's new k-mers."""
        nk = count_kmers(K, offsets)
        fl = np.zeros(max(nk, 1), np.uint8)
        ms = np.zeros(max(nk, 1), np.uint8)
        lib().orc_compactor_reads(self.h, int(canonical), K, _p(packed, u32p), _p(offsets, u64p),
                                  len(offsets) - 1, _p(fl, u8p), _p(ms, u8p))
        return fl[:nk], ms[:nk]

    def decision_masks(self, canonical, K, packed, offsets):
        nk = count_kmers(K, offsets)
        out = np.zeros(max(nk, 1), np.uint8)
        lib().orc_decision_masks(self.h, int(canonical), K, _p(packed, u32p), _p(offsets, u64p),
                                 len(offsets) - 1, _p(out, u8p))
        return out[:nk]


def count_kmers(K, offsets):
    offsets = np.ascontiguousarray(offsets, np.uint64)
    return int(lib().orc_count_kmers(K, _p(offsets, u64p), len(offsets) - 1))


def hash_reads(canonical, K, packed, offsets):
    nk = count_kmers(K, offsets)
    val = np.zeros(max(nk, 1), np.uint64)
    fw = np.zeros(max(nk, 1), np.uint64)
    rc = np.zeros(max(nk, 1), np.uint64)
    lib().orc_hash_reads(int(canonical), K, _p(packed, u32p), _p(offsets, u64p),
                         len(offsets) - 1, _p(val, u64p), _p(fw, u64p), _p(rc, u64p))
    return val[:nk], fw[:nk], rc[:nk]


def count_cells(canonical, K, packed, offsets, sizes, tables, lo, width, out=None, threads=1):
    """Touch counts (min 255) of cells [lo[j], lo[j] + width) of tables[j]
    over every k-mer of the batch, added to `out` (n_sel x width uint8,
    created when None): the final value of those cells is min(max, count)."""
    sizes = np.ascontiguousarray(sizes, np.uint64)
    sel = np.ascontiguousarray(tables, np.int32)
    lo = np.ascontiguousarray(lo, np.uint64)
    if out is None:
        out = np.zeros((len(sel), width), np.uint8)
    rc = lib().orc_count_cells(int(canonical), K, _p(packed, u32p), _p(offsets, u64p),
                               len(offsets) - 1, _p(sizes, u64p),
                               sel.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(sel),
                               _p(lo, u64p), width, _p(out, u8p), int(threads))
    if rc:
        raise MemoryError("orc_count_cells failed")
    return out


def pack_ascii(seqs, min_length=0):
    """FASTX-parser policy packer: returns (packed, offsets, n_skipped)."""
    data = b"".join(s.encode() if isinstance(s, str) else s for s in seqs)
    so = np.zeros(len(seqs) + 1, np.uint64)
    so[1:] = np.cumsum([len(s) for s in seqs])
    packed = np.zeros(len(data) // 16 + 2, np.uint32)
    offsets = np.zeros(len(seqs) + 1, np.uint64)
    skipped = ctypes.c_uint64()
    kept = lib().orc_pack_ascii(data, _p(so, u64p), len(seqs), min_length, _p(packed, u32p),
                                _p(offsets, u64p), ctypes.byref(skipped))
    return packed, offsets[:kept + 1].copy(), int(skipped.value)


def parse_fastx(text, min_length=0):
    """FastxParser<DNA_SIMPLE>::next over FASTA/FASTQ text until the end
    (kseq grammar).  Returns (kept sequences as a list of bytes, stats dict
    with n_parsed / n_skipped / n_dropped, status): status 0, or -2 when
    kseq reported differing sequence and quality lengths at record
    stats["invalid_record"] (the reads before it are kept)."""
    text = bytes(text)
    cap = len(text) + 1
    out = ctypes.create_string_buffer(cap)
    rec_cap = len(text) // 2 + 2
    off = np.zeros(rec_cap + 1, np.uint64)
    st = np.zeros(4, np.uint64)
    r = lib().orc_parse_fastx(text, len(text), min_length, out, cap, _p(off, u64p), rec_cap,
                              _p(st, u64p))
    if r == -5:
        raise RuntimeError("parse_fastx: output capacity")
    raw = out.raw
    # at an InvalidRead, the reads kept before it: every parsed read was kept or dropped
    kept = int(r) if r >= 0 else int(st[0] - st[2])
    seqs = [raw[int(off[i]):int(off[i + 1])] for i in range(kept)]
    stats = {"n_parsed": int(st[0]), "n_skipped": int(st[1]), "n_dropped": int(st[2]),
             "invalid_record": int(st[3]) if r == -2 else None}
    return seqs, stats, (0 if r >= 0 else int(r))


# ---- OXLI v4 table files ----------------------------------------------------
# The layout written by Storage::save and read by Storage::load:
#   "OXLI", version 4 (u8), file type (u8: 2 = BitStorage, bitstorage.cc:151-186;
#   1 = ByteStorage, bytestorage.cc:480-521; 7 = NibbleStorage,
#   nibblestorage.cc:132-166; codes from storage.hh:63-72),
#   [ByteStorage only: use_bigcount (u8)], ksize (u32), n_tables (u8),
#   occupied_bins (u64), then per table: table size in cells (u64) and the
#   table bytes (size/8+1, size, size/2+1), [ByteStorage only: the number of
#   bigcount entries (u64) and the entries].  Little-endian throughout.

OXLI_TYPE = {BIT: 2, BYTE: 1, NIBBLE: 7}


def oxli_bytes(kind, K, sizes, tables, n_occupied):
    """The file Storage::save writes for these tables (bytes)."""
    kind = KINDS[kind] if isinstance(kind, str) else kind
    out = [b"OXLI", bytes([4, OXLI_TYPE[kind]])]
    if kind == BYTE:
        out.append(b"\x00")
    out.append(np.array([K], "<u4").tobytes())
    out.append(bytes([len(sizes)]))
    out.append(np.array([n_occupied], "<u8").tobytes())
    for s, t in zip(sizes, tables):
        out.append(np.array([s], "<u8").tobytes())
        out.append(np.ascontiguousarray(t, np.uint8).tobytes())
    if kind == BYTE:
        out.append(np.zeros(1, "<u8").tobytes())
    return b"".join(out)


def parse_oxli(data):
    """Inverse of oxli_bytes: (kind, K, sizes, tables, n_occupied)."""
    data = bytes(data)
    if data[:4] != b"OXLI" or data[4] != 4:
        raise ValueError("not an OXLI v4 file")
    kind = {v: k for k, v in OXLI_TYPE.items()}[data[5]]
    pos = 6
    if kind == BYTE:
        pos += 1
    K = int(np.frombuffer(data, "<u4", 1, pos)[0])
    n = data[pos + 4]
    occ = int(np.frombuffer(data, "<u8", 1, pos + 5)[0])
    pos += 13
    sizes, tables = [], []
    for _ in range(n):
        s = int(np.frombuffer(data, "<u8", 1, pos)[0])
        nb = s // 8 + 1 if kind == BIT else s // 2 + 1 if kind == NIBBLE else s
        sizes.append(s)
        tables.append(np.frombuffer(data, np.uint8, nb, pos + 8).copy())
        pos += 8 + nb
    return kind, K, sizes, tables, occ


def update_from(tables_a, tables_b, occupied_a):
    """BitStorage::update_from (bitstorage.cc:103-137): byte-wise OR of B
    into A; occupied_bins grows by popcount(old ^ merged) over table 0."""
    if [len(t) for t in tables_a] != [len(t) for t in tables_b]:
        raise ValueError("both nodegraphs must have same table sizes")
    merged = [np.bitwise_or(a, b) for a, b in zip(tables_a, tables_b)]
    added = int(np.unpackbits(np.bitwise_xor(tables_a[0], merged[0])).sum())
    return merged, occupied_a + added
