"""Python mirror of goetia's dBG<Storage, Shifter> surface, backed by the GPU.

The reference exposes ``dBG[StorageType, ShifterType].build(storage, K)``
through cppyy (include/goetia/dbg.hh:39-438, goetia/pythonizors/
pythonize_dbg.py:4-53, pythonize_storage.py:5-41).  This module keeps those
names and argument meanings; every operation is a call into
libgoetia_gb300.so, which hashes, inserts and queries on the GPU.

Differences from the reference, all deliberate:
  * strings must hold only A/C/G/T.  The reference hashes other bytes
    silently (its own tests expect an exception and are marked xfail,
    tests/test_dbg.py:117-122, 215-221); here they raise
    InvalidSequenceException.
  * batch methods (``insert_packed`` and friends) take packed read batches
    and device buffers; they are the fast path.
"""
import ctypes
import os
import weakref

import numpy as np

from . import _lib
from .reads import PackedReads, pack_reads

_c = ctypes


# ---- hash value types (canonical.hh:30-147) ---------------------------------

class Hash(int):
    """Hash<uint64_t>: value() is the hash itself."""

    def value(self):
        return int(self)

    @property
    def hash(self):
        return int(self)


class Canonical(int):
    """Canonical<uint64_t>: min(fw_hash, rc_hash); sign() = fw < rc."""

    def __new__(cls, fw, rc):
        obj = int.__new__(cls, fw if fw < rc else rc)
        obj.fw_hash = int(fw)
        obj.rc_hash = int(rc)
        return obj

    def value(self):
        return int(self)

    def sign(self):
        return self.fw_hash < self.rc_hash


# ---- shifter and storage types ---------------------------------------------

class FwdLemireShifter:
    """HashShifter<LemireShifterPolicy<Hash<uint64_t>>> (hashshifter.hh:204)."""
    kind = _lib.FWD_LEMIRE
    hash_type = Hash


class CanLemireShifter:
    """HashShifter<LemireShifterPolicy<Canonical<uint64_t>>> (hashshifter.hh:205)."""
    kind = _lib.CAN_LEMIRE
    hash_type = Canonical


class _Handle:
    """Owns one C-ABI handle (gdbg_destroy on collection)."""

    def __init__(self, h):
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.gdbg_destroy(h)
            self.h = None


class _Storage:
    """Storage parameters plus, once a graph is built on it, the device
    tables: like the reference's shared_ptr<Storage> (dbg.hh:97-101), every
    dBG built on the same storage object shares its tables and counters."""
    kind = None
    is_counting = False
    is_probabilistic = True
    default_params = (1_000_000, 4)   # StorageTraits default_params (bitstorage.hh:75)

    def __init__(self, max_table=None, N=None, tablesizes=None):
        if tablesizes is not None:
            self.tablesizes = [int(x) for x in tablesizes]
        else:
            max_table = self.default_params[0] if max_table is None else max_table
            N = self.default_params[1] if N is None else N
            out = np.zeros(max(int(N), 1), np.uint64)
            got = _lib.c_u32()
            _lib.call("gdbg_primes_near", int(N), int(max_table),
                      out.ctypes.data_as(_lib.u64p), _c.byref(got))
            self.tablesizes = [int(v) for v in out[:got.value]]
        self.build_params = (max_table, N)
        self._anchor = None      # a handle on the device tables, once built
        self._graphs = weakref.WeakSet()   # the graphs built on it

    def _attach(self, h, shifter_kind, K):
        """Keep the tables of handle h alive with this storage object."""
        a = _c.c_void_p()
        _lib.call("gdbg_share_storage", h, shifter_kind, int(K), _c.byref(a))
        self._anchor = _Handle(a)

    @classmethod
    def build(cls, *args):
        """Storage::build(max_table, N) / build(params) / build()."""
        if len(args) == 1 and isinstance(args[0], tuple):
            args = args[0]
        return cls(*args)

    def get_tablesizes(self):
        return list(self.tablesizes)

    def _stats(self):
        # after the work queued on every graph built on the storage; empty
        # tables before the first one
        if self._anchor is None:
            return 0, 0
        for g in list(self._graphs):
            g.synchronize()
        u, o = _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_stats", self._anchor.h, _c.byref(u), _c.byref(o))
        return int(u.value), int(o.value)

    def n_unique_kmers(self):
        """k-mers that found a zero cell when inserted (bitstorage.hh:178-181)."""
        return self._stats()[0]

    def n_occupied(self):
        """Non-zero cells of table 0 (bitstorage.hh:173-176)."""
        return self._stats()[1]

    def estimated_fp(self):
        """(n_occupied / size_0) ^ n_tables (bitstorage.hh:183-187)."""
        return (self.n_occupied() / self.tablesizes[0]) ** len(self.tablesizes)

    def n_tables(self):
        return len(self.tablesizes)

    def describe(self):
        return (f"{type(self).__name__}\n- Params: {self.build_params}\n"
                f"- Probabilistic: {self.is_probabilistic}\n- Counting:      {self.is_counting}")


class BitStorage(_Storage):
    """Bloom filter, one bit per cell (bitstorage.hh:93-243)."""
    kind = _lib.BIT


class ByteStorage(_Storage):
    """8-bit saturating count-min sketch (bytestorage.hh:97-243)."""
    kind = _lib.BYTE
    is_counting = True


class NibbleStorage(_Storage):
    """4-bit saturating count-min sketch (nibblestorage.hh:89-232)."""
    kind = _lib.NIBBLE
    is_counting = True


def _p(a, t):
    return a.ctypes.data_as(t)


CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy


def _stream(s):
    """Stream argument for the C ABI: None -> the graph's own stream; 0 (the
    legacy default stream, e.g. torch's default) -> cudaStreamLegacy, since
    NULL means "the graph's own stream" there."""
    if s is None:
        return None
    s = int(s)
    return CUDA_STREAM_LEGACY if s == 0 else s


def _b(seq):
    if isinstance(seq, str):
        return seq.encode()
    return bytes(seq)


# ---- the graph -------------------------------------------------------------

class _dBGMeta(type):
    _cache = {}

    def __getitem__(cls, key):
        storage_type, shifter_type = key
        k = (storage_type, shifter_type)
        if k not in _dBGMeta._cache:
            name = f"dBG[{storage_type.__name__},{shifter_type.__name__}]"
            _dBGMeta._cache[k] = type(name, (dBGBase,),
                                      {"storage_type": storage_type,
                                       "shifter_type": shifter_type,
                                       "hash_type": shifter_type.hash_type})
        return _dBGMeta._cache[k]


class dBGBase:
    """One GPU-resident de Bruijn graph (dBG<Storage, Shifter>)."""
    storage_type = None
    shifter_type = None
    hash_type = None

    def __init__(self, handle, K, storage):
        self._h = handle
        self.K = int(K)
        self.storage = storage
        storage._graphs.add(self)
        self._cursor = None
        self._stream = None

    @classmethod
    def build(cls, storage, K):
        """dBG::build(storage, K) (dbg.hh:108-121)."""
        if isinstance(storage, type):
            storage = storage.build()
        h = _c.c_void_p()
        if storage._anchor is not None:
            # a storage already in use: share its tables
            _lib.call("gdbg_share_storage", storage._anchor.h, cls.shifter_type.kind, int(K),
                      _c.byref(h))
            return cls(h, K, storage)
        sizes = np.asarray(storage.tablesizes, np.uint64)
        _lib.call("gdbg_create_sized", storage.kind, cls.shifter_type.kind, int(K),
                  _p(sizes, _lib.u64p), len(sizes), _c.byref(h))
        storage._attach(h, cls.shifter_type.kind, K)
        return cls(h, K, storage)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.gdbg_destroy(h)
            self._h = None

    # -- storage-level -----------------------------------------------------
    def clone(self):
        """Empty graph on a new storage of the same table shape
        (dbg.hh:128-131, bitstorage.hh:136-138)."""
        h = _c.c_void_p()
        _lib.call("gdbg_clone", self._h, _c.byref(h))
        storage = type(self.storage)(tablesizes=self.storage.tablesizes)
        storage.build_params = self.storage.build_params
        storage._attach(h, self.shifter_type.kind, self.K)
        return type(self)(h, self.K, storage)

    shallow_clone = clone

    def reset(self):
        _lib.call("gdbg_reset", self._h)

    def n_unique(self):
        u, o = _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_stats", self._h, _c.byref(u), _c.byref(o))
        return int(u.value)

    def n_occupied(self):
        u, o = _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_stats", self._h, _c.byref(u), _c.byref(o))
        return int(o.value)

    def estimated_fp(self):
        """(n_occupied / size_0) ^ n_tables (bitstorage.hh:181-186)."""
        sizes = self.storage.tablesizes
        return (self.n_occupied() / sizes[0]) ** len(sizes)

    def table_bytes(self):
        out = np.zeros(len(self.storage.tablesizes), np.uint64)
        _lib.call("gdbg_table_bytes", self._h, _p(out, _lib.u64p))
        return [int(x) for x in out]

    def get_raw(self):
        """The tables in the reference's byte layout (dbg.hh:224-226)."""
        nb = self.table_bytes()
        flat = np.zeros(sum(nb), np.uint8)
        _lib.call("gdbg_get_tables", self._h, _p(flat, _lib.u8p), flat.size)
        out, pos = [], 0
        for n in nb:
            out.append(flat[pos:pos + n])
            pos += n
        return out

    def set_raw(self, tables):
        flat = np.ascontiguousarray(np.concatenate([np.asarray(t, np.uint8) for t in tables]))
        _lib.call("gdbg_set_tables", self._h, _p(flat, _lib.u8p), flat.size)

    def update_from(self, other):
        """BitStorage::update_from (bitstorage.cc:103-137), reached in the
        reference as graph.storage.update_from(other.storage): OR-merge
        other's Bit tables into this graph's."""
        _lib.call("gdbg_update_from", self._h, other._h)

    # -- OXLI files ----------------------------------------------------------
    def _gz(self, filename):
        # ByteStorageFile::save/load pick the gzip writer/reader by a ".gz"
        # suffix (bytestorage.cc:153-168, 640-657); Bit and Nibble files are
        # plain whatever the name.
        return self.storage_type is ByteStorage and str(filename).rsplit(".", 1)[-1] == "gz"

    def save(self, filename):
        """dBG::save (dbg.hh:396-398): the tables as an OXLI v4 file."""
        filename = os.fspath(filename)
        if not self._gz(filename):
            _lib.call("gdbg_save", self._h, filename.encode())
            return
        import gzip
        import shutil
        import tempfile
        with tempfile.NamedTemporaryFile(dir=os.path.dirname(os.path.abspath(filename)),
                                         delete=False) as tmp:
            plain = tmp.name
        try:
            _lib.call("gdbg_save", self._h, plain.encode())
            with open(plain, "rb") as src, gzip.open(filename, "wb") as dst:
                shutil.copyfileobj(src, dst, 16 << 20)
        finally:
            os.unlink(plain)

    def load(self, filename):
        """dBG::load (dbg.hh:400-403): replace the tables (and their sizes)
        by an OXLI v4 file's; K stays, the file's ksize is returned."""
        filename = os.fspath(filename)
        ks = _lib.c_u16()
        if not self._gz(filename):
            _lib.call("gdbg_load", self._h, filename.encode(), _c.byref(ks))
        else:
            import gzip
            import shutil
            import tempfile
            with tempfile.NamedTemporaryFile(delete=False) as tmp:
                plain = tmp.name
            try:
                try:
                    with gzip.open(filename, "rb") as src, open(plain, "wb") as dst:
                        shutil.copyfileobj(src, dst, 16 << 20)
                except (OSError, EOFError) as e:
                    raise _lib.GoetiaFileException(_lib.ERR_IO,
                                                   f"K-mer count file read error: {filename} {e}")
                _lib.call("gdbg_load", self._h, plain.encode(), _c.byref(ks))
            finally:
                os.unlink(plain)
        sizes = np.zeros(32, np.uint64)
        n = _lib.c_u16()
        _lib.call("gdbg_info", self._h, None, None, None, _c.byref(n))
        _lib.call("gdbg_get_tablesizes", self._h, _p(sizes, _lib.u64p))
        new = [int(x) for x in sizes[:n.value]]
        self.storage.tablesizes = new         # shared with every graph on it
        return int(ks.value)

    # -- hashing -----------------------------------------------------------
    def _wrap(self, value, fw, rc):
        if self.shifter_type is CanLemireShifter:
            return Canonical(fw, rc)
        return Hash(value)

    def hash(self, kmer):
        """HashShifter::hash of the first K symbols (hashshifter.hh:177-194)."""
        s = _b(kmer)
        v, fw, rc = _lib.c_u64(), _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_hash", self._h, s, len(s), _c.byref(v), _c.byref(fw), _c.byref(rc))
        return self._wrap(v.value, fw.value, rc.value)

    def hash_array(self, seq):
        """Hash values of every k-mer of seq as uint64 (value, fw, rc) arrays."""
        s = _b(seq)
        n = len(s) - self.K + 1
        if n < 1:
            raise _lib.SequenceLengthException(_lib.ERR_SEQUENCE_LENGTH,
                                               "Sequence must have length >= K")
        val, fw, rc = (np.zeros(n, np.uint64) for _ in range(3))
        _lib.call("gdbg_hashes", self._h, s, len(s), _p(val, _lib.u64p), _p(fw, _lib.u64p),
                  _p(rc, _lib.u64p))
        return val, fw, rc

    def hashes(self, sequence):
        """Generator over the k-mer hashes (pythonize_dbg.py:24-28)."""
        val, fw, rc = self.hash_array(sequence)
        for i in range(len(val)):
            yield self._wrap(int(val[i]), int(fw[i]), int(rc[i]))

    def get_hash_iter(self, sequence):
        return self.hashes(sequence)

    # -- single k-mers and hashes -------------------------------------------
    def _as_hash(self, item):
        if isinstance(item, (int, np.integer)):
            return int(item)
        s = _b(item)
        if len(s) < self.K:
            raise ValueError("k-mer shorter than K")
        return int(self.hash(s))

    def insert(self, item):
        """dBG::insert (dbg.hh:140-146): True when the k-mer was new."""
        h = np.array([self._as_hash(item)], np.uint64)
        out = np.zeros(1, np.uint8)
        _lib.call("gdbg_insert_hashes", self._h, _p(h, _lib.u64p), 1, _p(out, _lib.u8p))
        return bool(out[0])

    def query(self, item):
        """dBG::query (dbg.hh:171-177)."""
        h = np.array([self._as_hash(item)], np.uint64)
        out = np.zeros(1, np.int16)
        _lib.call("gdbg_query_hashes", self._h, _p(h, _lib.u64p), 1, _p(out, _lib.i16p))
        return int(out[0])

    def insert_and_query(self, item):
        """dBG::insert_and_query (dbg.hh:156-162): 1 if new, else the count."""
        new = self.insert(item)
        if self.storage.kind == _lib.BIT:
            return 1
        return 1 if new else self.query(item)

    def insert_hashes(self, hashes):
        """Insert hash values in order; returns the per-hash new flags."""
        h = np.ascontiguousarray(hashes, np.uint64)
        out = np.zeros(max(len(h), 1), np.uint8)
        _lib.call("gdbg_insert_hashes", self._h, _p(h, _lib.u64p), len(h), _p(out, _lib.u8p))
        return out[:len(h)].astype(bool)

    def query_hashes(self, hashes):
        h = np.ascontiguousarray(hashes, np.uint64)
        out = np.zeros(max(len(h), 1), np.int16)
        _lib.call("gdbg_query_hashes", self._h, _p(h, _lib.u64p), len(h), _p(out, _lib.i16p))
        return out[:len(h)]

    add = insert
    get = query

    # -- sequences ---------------------------------------------------------
    def insert_sequence(self, sequence, *out):
        """dBG::insert_sequence overloads (dbg.hh:249-318).

        insert_sequence(seq) -> number of k-mers
        insert_sequence(seq, n_new) with a ctypes.c_uint64 -> fills n_new
        insert_sequence(seq, hashes) with a list -> appends the k-mer hashes
        insert_sequence(seq, new_kmers) with a set -> adds the new k-mers' hashes
        insert_sequence(seq, hashes, counts) -> appends hashes and
            post-insertion counts (insert_and_query per k-mer, in order)
        """
        s = _b(sequence)
        if len(out) == 2:
            hashes, counts = out
            hs = self.hashes(s)
            hashes.extend(hs)
            counts.extend(self.insert_and_query_sequence(s))
            return len(s) - self.K + 1
        if len(out) == 1 and isinstance(out[0], (list, set)):
            vals = list(self.hashes(s))
            if isinstance(out[0], list):
                self.insert_hashes(np.array([int(v) for v in vals], np.uint64))
                out[0].extend(vals)
            else:
                new = self.insert_hashes(np.array([int(v) for v in vals], np.uint64))
                out[0].update(v for v, n in zip(vals, new) if n)
            return len(s) - self.K + 1
        nk, nn = _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_insert_sequence", self._h, s, len(s), _c.byref(nk), _c.byref(nn))
        if len(out) == 1:
            out[0].value = nn.value
        return int(nk.value)

    def insert_sequence_new(self, sequence):
        """(n_kmers, n_new) for one sequence."""
        s = _b(sequence)
        nk, nn = _lib.c_u64(), _lib.c_u64()
        _lib.call("gdbg_insert_sequence", self._h, s, len(s), _c.byref(nk), _c.byref(nn))
        return int(nk.value), int(nn.value)

    def insert_and_query_sequence(self, sequence):
        """Post-insertion counts, k-mer by k-mer (dbg.hh:327-340)."""
        s = _b(sequence)
        n = len(s) - self.K + 1
        if n < 1:
            raise _lib.SequenceLengthException(_lib.ERR_SEQUENCE_LENGTH,
                                               "Sequence must have length >= K")
        c = np.zeros(n, np.int16)
        _lib.call("gdbg_insert_and_query_sequence", self._h, s, len(s), _p(c, _lib.i16p), None)
        return [int(x) for x in c]

    def query_sequence(self, sequence, counts=None, hashes=None):
        """dBG::query_sequence (dbg.hh:349-394)."""
        s = _b(sequence)
        n = len(s) - self.K + 1
        if n < 1:
            raise _lib.SequenceLengthException(_lib.ERR_SEQUENCE_LENGTH,
                                               "Sequence must have length >= K")
        c = np.zeros(n, np.int16)
        h = np.zeros(n, np.uint64)
        _lib.call("gdbg_query_sequence", self._h, s, len(s), _p(c, _lib.i16p), _p(h, _lib.u64p))
        if counts is not None:
            counts.extend(int(x) for x in c)
            if hashes is not None:
                hashes.extend(self.hashes(s))
            return None
        return [int(x) for x in c]

    # -- neighbours / decision k-mers -----------------------------------------
    def neighbor_masks(self, sequence):
        """uint8 per k-mer: bit i = left "ACGT"[i] present, bit 4+i = right."""
        s = _b(sequence)
        n = len(s) - self.K + 1
        if n < 1:
            raise _lib.SequenceLengthException(_lib.ERR_SEQUENCE_LENGTH,
                                               "Sequence must have length >= K")
        m = np.zeros(n, np.uint8)
        _lib.call("gdbg_neighbor_masks", self._h, s, len(s), _p(m, _lib.u8p))
        return m

    def set_cursor(self, kmer):
        """HashExtender::set_cursor (hashextender.hh:178-197)."""
        s = _b(kmer)
        if len(s) < self.K:
            raise _lib.InvalidSequenceException(_lib.ERR_INVALID_SEQUENCE,
                                                "Sequence must at least length K")
        self._cursor = s[:self.K]
        return self.hash(self._cursor)

    def get_cursor(self):
        return self._cursor.decode() if self._cursor is not None else None

    def _cursor_mask(self):
        if self._cursor is None:
            raise _lib.GoetiaError(_lib.ERR_INVALID_ARG, "UninitializedShifterException")
        return int(self.neighbor_masks(self._cursor)[0])

    def in_degree(self):
        """Present left extensions of the cursor (unitig_walker.hh:322-325)."""
        return bin(self._cursor_mask() & 15).count("1")

    def out_degree(self):
        """Present right extensions of the cursor (unitig_walker.hh:327-330)."""
        return bin(self._cursor_mask() >> 4).count("1")

    def degree(self):
        return self.in_degree() + self.out_degree()

    def left_degree(self, kmer):
        self.set_cursor(kmer)
        return self.in_degree()

    def right_degree(self, kmer):
        self.set_cursor(kmer)
        return self.out_degree()

    def left_extensions(self):
        """Hashes of "ACGT"[i] + cursor[:-1] (hashextender.hh:352-364)."""
        c = self._cursor.decode()
        return [self.hash(s + c[:-1]) for s in "ACGT"]

    def right_extensions(self):
        """Hashes of cursor[1:] + "ACGT"[i] (hashextender.hh:386-396)."""
        c = self._cursor.decode()
        return [self.hash(c[1:] + s) for s in "ACGT"]

    def is_decision_kmer(self, node=None):
        """in_degree > 1 or out_degree > 1 (unitig_walker.hh:1003-1023)."""
        if node is not None:
            self.set_cursor(node)
        m = self._cursor_mask()
        return bin(m & 15).count("1") > 1 or bin(m >> 4).count("1") > 1

    def find_decision_kmers(self, sequence):
        """(positions, hashes) of decision k-mers (unitig_walker.hh:1025-1045)."""
        m = self.neighbor_masks(sequence)
        lo = np.unpackbits((m & 15)[:, None], axis=1).sum(1)
        hi = np.unpackbits((m >> 4)[:, None], axis=1).sum(1)
        pos = np.nonzero((lo > 1) | (hi > 1))[0]
        hs = list(self.hashes(sequence))
        return [int(p) for p in pos], [hs[p] for p in pos]

    # -- packed batches (host numpy buffers) ------------------------------------
    @staticmethod
    def _packed(reads):
        if isinstance(reads, PackedReads):
            return reads
        return pack_reads(reads)

    def insert_packed(self, reads):
        """insert_sequence for every read in order; per-read new counts."""
        r = self._packed(reads)
        n_new = np.zeros(max(r.n_reads, 1), np.uint64)
        nk = _lib.c_u64()
        _lib.call("gdbg_insert_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(n_new, _lib.u64p), _c.byref(nk))
        return n_new[:r.n_reads]

    def compactor_query(self, sequence):
        """The compactor's per-k-mer query of one sequence (compactor.hh:
        346-466) against the storage as it is: (new, seen, masks) arrays --
        new = query() == 0, seen = already in the sequence's new-k-mer set,
        masks = neighbour masks over the storage plus the sequence's new
        k-mers (filter_nodes with extras, unitig_walker.hh:457-469)."""
        s = _b(sequence)
        n = len(s) - self.K + 1
        if n < 1:
            raise _lib.SequenceLengthException(_lib.ERR_SEQUENCE_LENGTH,
                                               "Sequence must have length >= K")
        fl = np.zeros(n, np.uint8)
        ms = np.zeros(n, np.uint8)
        _lib.call("gdbg_compactor_sequence", self._h, s, len(s), _p(fl, _lib.u8p), _p(ms, _lib.u8p))
        return (fl & 1).astype(bool), (fl & 2).astype(bool), ms

    def compactor_query_packed(self, reads):
        """compactor_query for every read of a batch (each against the
        storage as it is before the call): flattened (flags, masks), flags
        bit 0 = new, bit 1 = seen."""
        r = self._packed(reads)
        n = r.n_kmers(self.K)
        fl = np.zeros(max(n, 1), np.uint8)
        ms = np.zeros(max(n, 1), np.uint8)
        _lib.call("gdbg_compactor_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(fl, _lib.u8p), _p(ms, _lib.u8p))
        return fl[:n], ms[:n]

    def insert_and_query_packed(self, reads):
        """insert_and_query_sequence for every read in order: (flattened
        counts, per-read new counts), equal to the sequential calls."""
        r = self._packed(reads)
        n = r.n_kmers(self.K)
        c = np.zeros(max(n, 1), np.int16)
        n_new = np.zeros(max(r.n_reads, 1), np.uint64)
        _lib.call("gdbg_insert_and_query_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(c, _lib.i16p), _p(n_new, _lib.u64p))
        return c[:n], n_new[:r.n_reads]

    def query_packed(self, reads):
        r = self._packed(reads)
        c = np.zeros(max(r.n_kmers(self.K), 1), np.int16)
        _lib.call("gdbg_query_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(c, _lib.i16p))
        return c[:r.n_kmers(self.K)]

    def hashes_packed(self, reads):
        r = self._packed(reads)
        n = r.n_kmers(self.K)
        val, fw, rc = (np.zeros(max(n, 1), np.uint64) for _ in range(3))
        _lib.call("gdbg_hashes_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(val, _lib.u64p), _p(fw, _lib.u64p),
                  _p(rc, _lib.u64p))
        return val[:n], fw[:n], rc[:n]

    def neighbor_masks_packed(self, reads):
        r = self._packed(reads)
        n = r.n_kmers(self.K)
        m = np.zeros(max(n, 1), np.uint8)
        _lib.call("gdbg_neighbor_masks_batch", self._h, _p(r.packed, _lib.u32p), r.packed.size,
                  _p(r.offsets, _lib.u64p), r.n_reads, _p(m, _lib.u8p))
        return m[:n]

    # -- device buffers (torch tensors or raw pointers) ---------------------------
    def set_stream(self, stream):
        """Run this graph's work on a CUDA stream (a cudaStream_t value or None)."""
        _lib.call("gdbg_set_stream", self._h, _stream(stream))
        self._stream = stream

    def synchronize(self):
        _lib.call("gdbg_synchronize", self._h)

    def insert_device(self, packed_ptr, packed_words, offsets_ptr, n_reads, n_kmers=None,
                      n_new_ptr=None, stream=None):
        """Asynchronous batch insert from device pointers (see gdbg_insert_batch_device)."""
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_insert_batch_device", self._h, packed_ptr, int(packed_words), offsets_ptr,
                  int(n_reads), hint, n_new_ptr, _stream(stream))

    def insert_and_query_device(self, packed_ptr, packed_words, offsets_ptr, n_reads, counts_ptr,
                                n_new_ptr=None, n_kmers=None, stream=None):
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_insert_and_query_batch_device", self._h, packed_ptr, int(packed_words),
                  offsets_ptr, int(n_reads), hint, counts_ptr, n_new_ptr, _stream(stream))

    def insert_async(self, packed_ptr, packed_words, offsets_ptr, n_reads, n_kmers, n_new_ptr,
                     stream=None):
        """gdbg_insert_batch_async: host (pinned) buffers in and out, all work
        queued on `stream`; returns at once.  n_kmers None: the call counts
        the k-mers from the host offsets."""
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_insert_batch_async", self._h, packed_ptr, int(packed_words), offsets_ptr,
                  int(n_reads), hint, n_new_ptr, _stream(stream))

    def reserve_staging(self, max_words, max_reads):
        _lib.call("gdbg_reserve_staging", self._h, int(max_words), int(max_reads))

    def query_device(self, packed_ptr, packed_words, offsets_ptr, n_reads, counts_ptr,
                     n_kmers=None, stream=None):
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_query_batch_device", self._h, packed_ptr, int(packed_words), offsets_ptr,
                  int(n_reads), hint, counts_ptr, _stream(stream))

    def neighbor_masks_device(self, packed_ptr, packed_words, offsets_ptr, n_reads, masks_ptr,
                              n_kmers=None, stream=None):
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_neighbor_masks_batch_device", self._h, packed_ptr, int(packed_words),
                  offsets_ptr, int(n_reads), hint, masks_ptr, _stream(stream))

    def hashes_device(self, packed_ptr, packed_words, offsets_ptr, n_reads, values_ptr,
                      fw_ptr=None, rc_ptr=None, n_kmers=None, stream=None):
        hint = (1 << 64) - 1 if n_kmers is None else int(n_kmers)
        _lib.call("gdbg_hashes_batch_device", self._h, packed_ptr, int(packed_words), offsets_ptr,
                  int(n_reads), hint, values_ptr, fw_ptr, rc_ptr, _stream(stream))

    # -- tuning / diagnostics -----------------------------------------------
    def set_insert_schedule(self, window_kmers=0, kmers_per_thread=0):
        _lib.call("gdbg_set_insert_schedule", self._h, int(window_kmers), int(kmers_per_thread))

    PATHS = {"persistent": _lib.PATH_PERSISTENT, "windowed": _lib.PATH_WINDOWED,
             "bucketed": _lib.PATH_BUCKETED, "auto": _lib.PATH_AUTO,
             "bucketed_ordered": _lib.PATH_BUCKETED_ORDERED,
             True: _lib.PATH_PERSISTENT, False: _lib.PATH_WINDOWED}

    def set_insert_path(self, path="auto"):
        """Batch insert implementation: "persistent", "windowed", "bucketed",
        "bucketed_ordered" or "auto" (True / False mean persistent / windowed)."""
        _lib.call("gdbg_set_insert_path", self._h, self.PATHS[path])
        self._path = path

    def insert_path(self):
        """The path last set with set_insert_path ("auto" by default)."""
        return getattr(self, "_path", "auto")

    def set_bucket_bits(self, log2_cells=0):
        """Cells per bucket (log2) of the bucketed paths; 0 = their default
        (adaptive for "bucketed", 64 KB of table for "bucketed_ordered")."""
        _lib.call("gdbg_set_bucket_bits", self._h, int(log2_cells))

    def insert_schedule(self):
        w, k = _lib.c_u32(), _lib.c_u32()
        _lib.call("gdbg_get_insert_schedule", self._h, _c.byref(w), _c.byref(k))
        return int(w.value), int(k.value)

    def device_status(self):
        s = _lib.c_u32()
        _lib.call("gdbg_device_status", self._h, _c.byref(s))
        return int(s.value)

    def set_wait_limits(self, barrier_polls=0, copy_polls=0):
        """Poll limits of the bounded device waits (0 = default, 2^24): the
        persistent insert's grid barrier and the bucketed insert's first wait
        on each bulk copy.  A wait that runs out ends its kernel early and the
        next synchronising call raises GoetiaError (GDBG_ERR_DEVICE)."""
        _lib.call("gdbg_set_wait_limits", self._h, int(barrier_polls), int(copy_polls))

    def reserve(self, max_reads, max_kmers):
        """Grow the insert scratch for batches up to this size now."""
        _lib.call("gdbg_reserve", self._h, int(max_reads), int(max_kmers))

    def set_profiling(self, on=True):
        """Bracket each insert stage with CUDA events (see stage_times)."""
        _lib.call("gdbg_set_profiling", self._h, 1 if on else 0)

    def stage_times(self):
        """{stage: (total_ms, launches)} since the last call (synchronises)."""
        names = _c.create_string_buffer(4096)
        ms = (_c.c_double * 64)()
        cnt = (_c.c_uint64 * 64)()
        n = _lib.c_u32()
        _lib.call("gdbg_stage_times", self._h, names, 4096, ms, cnt, 64, _c.byref(n))
        keys = names.value.decode().split(",") if n.value else []
        return {k: (ms[i], int(cnt[i])) for i, k in enumerate(keys[:64])}

    def launch_count(self):
        n = _lib.c_u64()
        _lib.call("gdbg_launch_count", self._h, _c.byref(n))
        return int(n.value)


class dBG(metaclass=_dBGMeta):
    """``dBG[StorageType, ShifterType]`` -> graph class with ``build(storage, K)``."""
