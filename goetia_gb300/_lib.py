"""ctypes binding of libgoetia_gb300.so (the C ABI in include/goetia_gb300.h).

The shared library is the product: every hash, insert, query and mask in
this package runs through it on the GPU.  Loading fails loudly when it is
missing; there is no other code path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgoetia_gb300.so")

OK = 0
ERR_INVALID_ARG = 1
ERR_SEQUENCE_LENGTH = 2
ERR_INVALID_SEQUENCE = 3
ERR_CUDA = 4
ERR_OOM = 5
ERR_DEVICE = 6
ERR_IO = 7
ERR_UNSUPPORTED = 8

BIT, BYTE, NIBBLE = 0, 1, 2
FWD_LEMIRE, CAN_LEMIRE = 0, 1
PATH_PERSISTENT, PATH_WINDOWED, PATH_BUCKETED, PATH_AUTO, PATH_BUCKETED_ORDERED = 0, 1, 2, 3, 4

c_u64 = ctypes.c_uint64
c_u32 = ctypes.c_uint32
c_u16 = ctypes.c_uint16
c_int = ctypes.c_int
c_vp = ctypes.c_void_p
c_cp = ctypes.c_char_p
P = ctypes.POINTER
u64p, u32p, u16p, u8p, i16p, intp = (P(c_u64), P(c_u32), P(c_u16), P(ctypes.c_uint8),
                                      P(ctypes.c_int16), P(c_int))

# name -> argtypes (every entry point returns int)
SIGNATURES = {
    "gdbg_primes_near": [c_u32, c_u64, u64p, u32p],
    "gdbg_create": [c_int, c_int, c_u16, c_u64, c_u16, P(c_vp)],
    "gdbg_create_sized": [c_int, c_int, c_u16, u64p, c_u16, P(c_vp)],
    "gdbg_destroy": [c_vp],
    "gdbg_clone": [c_vp, P(c_vp)],
    "gdbg_share_storage": [c_vp, c_int, c_u16, P(c_vp)],
    "gdbg_reset": [c_vp],
    "gdbg_info": [c_vp, intp, intp, u16p, u16p],
    "gdbg_get_tablesizes": [c_vp, u64p],
    "gdbg_table_bytes": [c_vp, u64p],
    "gdbg_get_tables": [c_vp, u8p, c_u64],
    "gdbg_set_tables": [c_vp, u8p, c_u64],
    "gdbg_stats": [c_vp, u64p, u64p],
    "gdbg_save": [c_vp, c_cp],
    "gdbg_load": [c_vp, c_cp, u16p],
    "gdbg_update_from": [c_vp, c_vp],
    "gdbg_set_stream": [c_vp, c_vp],
    "gdbg_synchronize": [c_vp],
    "gdbg_hash": [c_vp, c_cp, c_u64, u64p, u64p, u64p],
    "gdbg_insert_sequence": [c_vp, c_cp, c_u64, u64p, u64p],
    "gdbg_query_sequence": [c_vp, c_cp, c_u64, i16p, u64p],
    "gdbg_insert_and_query_sequence": [c_vp, c_cp, c_u64, i16p, u64p],
    "gdbg_hashes": [c_vp, c_cp, c_u64, u64p, u64p, u64p],
    "gdbg_insert_hashes": [c_vp, u64p, c_u64, u8p],
    "gdbg_query_hashes": [c_vp, u64p, c_u64, i16p],
    "gdbg_neighbor_masks": [c_vp, c_cp, c_u64, u8p],
    "gdbg_pack_reads_device": [c_vp, c_vp, c_u64, c_u32, c_vp, c_u64, c_vp, u64p, u64p, c_vp],
    "gdbg_parse_fastx_device": [c_vp, c_u64, c_u32, c_vp, c_u64, c_vp, c_u64, u64p, c_vp],
    "gdbg_pack_reads": [c_cp, u64p, c_u64, c_u32, u32p, c_u64, u64p, u64p, u64p],
    "gdbg_pack_codes": [u8p, c_u64, u32p],
    "gdbg_insert_batch": [c_vp, u32p, c_u64, u64p, c_u64, u64p, u64p],
    "gdbg_query_batch": [c_vp, u32p, c_u64, u64p, c_u64, i16p],
    "gdbg_insert_and_query_batch": [c_vp, u32p, c_u64, u64p, c_u64, i16p, u64p],
    "gdbg_hashes_batch": [c_vp, u32p, c_u64, u64p, c_u64, u64p, u64p, u64p],
    "gdbg_neighbor_masks_batch": [c_vp, u32p, c_u64, u64p, c_u64, u8p],
    "gdbg_compactor_sequence": [c_vp, c_cp, c_u64, u8p, u8p],
    "gdbg_compactor_batch": [c_vp, u32p, c_u64, u64p, c_u64, u8p, u8p],
    "gdbg_compactor_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp, c_vp],
    "gdbg_insert_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp],
    "gdbg_insert_batch_async": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp],
    "gdbg_reserve_staging": [c_vp, c_u64, c_u64],
    "gdbg_query_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp],
    "gdbg_insert_and_query_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp,
                                           c_vp],
    "gdbg_hashes_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp, c_vp, c_vp],
    "gdbg_neighbor_masks_batch_device": [c_vp, c_vp, c_u64, c_vp, c_u64, c_u64, c_vp, c_vp],
    "gdbg_set_insert_schedule": [c_vp, c_u32, c_u32],
    "gdbg_get_insert_schedule": [c_vp, u32p, u32p],
    "gdbg_set_insert_path": [c_vp, c_int],
    "gdbg_set_bucket_bits": [c_vp, c_u32],
    "gdbg_device_status": [c_vp, u32p],
    "gdbg_set_wait_limits": [c_vp, c_u32, c_u32],
    "gdbg_server_create": [c_int, c_int, c_u16, c_u16, c_u64, c_u32, c_u32, P(c_vp)],
    "gdbg_server_stream": [c_vp, c_u64, c_u64, c_u64, c_u64],
    "gdbg_server_submit": [c_vp, c_u64, c_vp, c_u64, c_vp, c_u64, c_u64, ctypes.c_double, c_vp,
                           c_u64],
    "gdbg_server_finish": [c_vp, c_u64],
    "gdbg_server_stream_bytes": [c_vp, c_u64, P(c_u64)],
    "gdbg_server_start": [c_vp],
    "gdbg_server_wait": [c_vp, ctypes.c_double],
    "gdbg_server_poll": [c_vp, c_vp, c_vp, c_vp, c_vp, c_u64, P(c_u64)],
    "gdbg_server_stats": [c_vp, c_vp],
    "gdbg_server_destroy": [c_vp],
    "gdbg_noalloc_table_layout": [c_int, u64p, c_u16, u64p],
    "gdbg_insert_batch_noalloc": [c_int, c_int, c_u16, u64p, c_u16, c_vp, c_vp, c_u64, c_vp,
                                  c_u64, c_vp, c_vp, c_vp],
    "gdbg_launch_count": [c_vp, u64p],
    "gdbg_set_profiling": [c_vp, c_int],
    "gdbg_reserve": [c_vp, c_u64, c_u64],
    "gdbg_stage_times": [c_vp, c_cp, c_u64, P(ctypes.c_double), u64p, c_u32, u32p],
}

_lib = None


class ServerReport(ctypes.Structure):
    """gdbg_server_report (include/goetia_gb300.h)."""
    _fields_ = [(n, c_u64) for n in ("chunks_submitted", "chunks_done", "chunks_failed",
                                      "kmers_done", "streams", "streams_admitted",
                                      "admission_waits", "lazy_frees", "peak_hbm_bytes")] + \
               [(n, ctypes.c_double) for n in ("first_dispatch_s", "last_done_s", "admit_s_max",
                                                "admit_s_total", "dispatch_s_max",
                                                "dispatch_s_total")] + \
               [("device_status", c_u32)]


class GoetiaError(RuntimeError):
    """A C-ABI call failed; `code` is the GDBG_ERR_* status."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class SequenceLengthException(GoetiaError, ValueError):
    """Sequence shorter than K (kmeriterator.hh:57-59)."""


class InvalidSequenceException(GoetiaError, ValueError):
    """Symbol outside DNA_SIMPLE, or a k-mer shorter than K (alphabets.hh:41-56)."""


class GoetiaFileException(GoetiaError, OSError):
    """Table file missing, truncated or of the wrong kind (goetia.hh
    GoetiaFileException, raised by Storage::load, bitstorage.cc:188-307)."""


def load():
    """Load the in-tree shared library (build it with goetia_gb300.build first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m goetia_gb300.build` "
                          "(nvcc, sm_103a) before using goetia_gb300")
    L = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = c_int
    L.gdbg_last_error.restype = c_cp
    L.gdbg_last_error.argtypes = []
    L.gdbg_version.restype = c_cp
    L.gdbg_version.argtypes = []
    L.gdbg_server_last_error.restype = c_cp
    L.gdbg_server_last_error.argtypes = [c_vp]
    _lib = L
    return L


def check(rc):
    if rc == OK:
        return
    msg = load().gdbg_last_error().decode(errors="replace")
    if rc == ERR_SEQUENCE_LENGTH:
        raise SequenceLengthException(rc, msg)
    if rc == ERR_INVALID_SEQUENCE:
        raise InvalidSequenceException(rc, msg)
    if rc == ERR_OOM:
        raise MemoryError(msg)
    if rc == ERR_IO:
        raise GoetiaFileException(rc, msg)
    raise GoetiaError(rc, msg)


def call(name, *args):
    check(getattr(load(), name)(*args))
