"""goetia_gb300: GB300-native (sm_103a) hot path of goetia's dBG.

Canonical / forward cyclic rolling k-mer hashing, batched insert into and
query of the Bit / Byte / Nibble storages, and neighbour (decision-node)
masks, all computed by hand-written CUDA kernels behind the C ABI in
include/goetia_gb300.h.  The Python surface mirrors goetia's
``dBG[Storage, Shifter]`` API (include/goetia/dbg.hh).
"""
from ._lib import (GoetiaError, GoetiaFileException, InvalidSequenceException,
                   SequenceLengthException, load)
from .dbg import (BitStorage, ByteStorage, CanLemireShifter, Canonical, FwdLemireShifter, Hash,
                  NibbleStorage, dBG)
from .reads import PackedReads, from_codes, pack_codes, pack_reads

__all__ = [
    "BitStorage", "ByteStorage", "NibbleStorage", "FwdLemireShifter", "CanLemireShifter",
    "Hash", "Canonical", "dBG", "PackedReads", "pack_reads", "pack_codes", "from_codes",
    "GoetiaError", "GoetiaFileException", "InvalidSequenceException", "SequenceLengthException", "load",
]
