"""The C ABI library: builds, loads, exports every declared symbol, and its
host-only helpers (table sizing, read packing) agree with the oracle.
CPU only -- nothing here launches a kernel."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from goetia_gb300 import _lib, build, reads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared():
    out = set()
    for h in HEADERS:
        text = open(h).read()
        out |= set(re.findall(r"^\s*(?:int|const char\*)\s+(gdbg_\w+)\s*\(", text, re.M))
    return out


def test_header_declares_entry_points():
    names = declared()
    assert "gdbg_insert_batch" in names and "gdbg_create" in names
    assert len(names) > 30


def test_library_exports_every_declared_symbol(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_binding_table_matches_header():
    names = declared() - {"gdbg_last_error", "gdbg_version", "gdbg_server_last_error"}
    assert set(_lib.SIGNATURES) <= declared()
    missing = names - set(_lib.SIGNATURES)
    assert not missing, missing


def test_version(lib):
    assert b"sm_103a" in lib.gdbg_version()


@pytest.mark.parametrize("n,x", [(4, 4194304), (4, 1 << 30), (3, 10), (1, 1), (4, 1000), (5, 12)])
def test_primes_near(lib, n, x):
    out = np.zeros(n, np.uint64)
    got = ctypes.c_uint32()
    _lib.call("gdbg_primes_near", n, x, out.ctypes.data_as(_lib.u64p), ctypes.byref(got))
    assert [int(v) for v in out[:got.value]] == oracle.primes(n, x)


def test_pack_reads_matches_parser_policy():
    rng = np.random.default_rng(3)
    alphabet = np.array(list("ACGTacgtNnXY"))
    seqs = []
    for i in range(300):
        L = int(rng.integers(0, 70))
        p = np.r_[np.full(8, 0.12), np.full(4, 0.01)]
        seqs.append("".join(rng.choice(alphabet, L, p=p / p.sum())))
    for min_len in (0, 20):
        got = reads.pack_reads(seqs, min_length=min_len)
        ref_packed, ref_off, ref_skip = oracle.pack_ascii(seqs, min_length=min_len)
        assert got.n_skipped == ref_skip
        assert np.array_equal(got.offsets, ref_off)
        n_words = (int(ref_off[-1]) + 15) // 16
        assert np.array_equal(got.packed[:n_words], ref_packed[:n_words])


def test_pack_codes_layout():
    rng = np.random.default_rng(4)
    c = rng.integers(0, 4, 1000, dtype=np.uint8)
    p = reads.pack_codes(c)
    j = np.arange(1000)
    assert np.array_equal((p[j >> 4] >> (2 * (j & 15)).astype(np.uint32)) & 3, c)


def test_numpy_packer_equals_library_packer():
    """synth.pack_codes_np (numpy alone, for runs that must not load the GPU
    library) gives the library packer's words, padding included."""
    from goetia_gb300 import synth
    rng = np.random.default_rng(5)
    for n in (0, 1, 15, 16, 17, 33, 1000, 150 * 1001):
        c = rng.integers(0, 4, n, dtype=np.uint8)
        a, b = synth.pack_codes_np(c), reads.pack_codes(c)
        assert a.dtype == np.uint32 and np.array_equal(a, b)
    rows = rng.integers(0, 4, (300, 150), dtype=np.uint8)
    pa, pb = synth.rows_to_packed(rows, native=False), synth.rows_to_packed(rows)
    assert np.array_equal(pa.packed, pb.packed) and np.array_equal(pa.offsets, pb.offsets)


def test_from_codes_and_kmer_count():
    rng = np.random.default_rng(9)
    rows = [rng.integers(0, 4, L, dtype=np.uint8) for L in (0, 5, 31, 32, 150)]
    pr = reads.from_codes(rows)
    assert pr.n_reads == 5 and pr.n_bases == 218
    assert pr.n_kmers(31) == 0 + 0 + 1 + 2 + 120   # short and empty reads count zero
    flat = np.concatenate(rows)
    j = np.arange(len(flat))
    assert np.array_equal((pr.packed[j >> 4] >> (2 * (j & 15)).astype(np.uint32)) & 3, flat)
    grid = rng.integers(0, 4, (7, 40), dtype=np.uint8)
    pg = reads.from_codes(grid)
    assert [int(v) for v in pg.offsets] == [40 * i for i in range(8)]
    assert pg.n_kmers(21) == 7 * 20
    assert reads.codes_to_str(reads.str_to_codes("GATTACA")) == "GATTACA"


def test_storage_params_mirror():
    from goetia_gb300 import BitStorage, ByteStorage, NibbleStorage
    s = BitStorage.build(4194304, 4)
    assert s.get_tablesizes() == [4194301, 4194287, 4194277, 4194271]
    assert BitStorage.build().get_tablesizes() == oracle.primes(4, 1_000_000)
    assert ByteStorage.is_counting and NibbleStorage.is_counting and not BitStorage.is_counting


def test_cpp_wrapper_compiles_and_links(lib, tmp_path):
    """include/goetia_gb300.hpp (the reference-signature C++ front end) builds
    and links against the library (not run: no GPU here)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "t.cc"
    src.write_text(
        '#include "goetia_gb300.hpp"\n'
        "using namespace goetia_gb300;\n"
        "int main() {\n"
        "  auto g = GpuDBG<ByteStorage, CanLemireShifter>::build(100000, 4, 31);\n"
        "  uint64_t n_new = 0;\n"
        '  g->insert_sequence(std::string(40, \'A\'), n_new);\n'
        '  auto c = g->query_sequence(std::string(40, \'A\'));\n'
        "  return (int)c.size() + (int)n_new;\n"
        "}\n")
    libdir = os.path.join(ROOT, "goetia_gb300")
    subprocess.check_call([gxx, "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src),
                           "-o", str(tmp_path / "t"), "-L", libdir, "-l:libgoetia_gb300.so",
                           "-Wl,-rpath-link,/usr/local/cuda/lib64",
                           "-L/usr/local/cuda/lib64", "-lcudart"])
