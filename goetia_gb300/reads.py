"""Packed read batches: the 2-bit base stream plus base offsets.

``pack_reads`` applies goetia's FASTX-parser policy for DNA_SIMPLE
(FastxParser::next, include/goetia/parsing/readers.hh:150-219): lowercase
acgt are upper-cased, reads holding any other symbol or shorter than
``min_length`` are dropped and counted.
"""
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class PackedReads:
    packed: np.ndarray    # uint32, 16 bases per word
    offsets: np.ndarray   # uint64, n_reads + 1 base offsets
    n_skipped: int = 0

    @property
    def n_reads(self):
        return len(self.offsets) - 1

    @property
    def n_bases(self):
        return int(self.offsets[-1]) if len(self.offsets) else 0

    def n_kmers(self, K):
        lens = np.diff(self.offsets.astype(np.int64))
        return int(np.maximum(lens - K + 1, 0).sum())

    def slice(self, r0, r1):
        """Reads r0 .. r1-1 as a PackedReads over the same words (no copy of
        the bases): the words from the one holding read r0's first base, the
        offsets shifted to match."""
        b0 = int(self.offsets[r0])
        w0 = b0 // 16
        w1 = (int(self.offsets[r1]) + 15) // 16 + 1
        off = (self.offsets[r0:r1 + 1] - np.uint64(16 * w0)).astype(np.uint64)
        return PackedReads(self.packed[w0:min(w1, len(self.packed))], off, 0)


def _p(a, t):
    return a.ctypes.data_as(t)


def pack_reads(seqs, min_length=0):
    """Text reads (str or bytes) -> PackedReads, dropping invalid reads."""
    enc = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    data = b"".join(enc)
    so = np.zeros(len(enc) + 1, np.uint64)
    if enc:
        so[1:] = np.cumsum([len(s) for s in enc], dtype=np.uint64)
    words = len(data) // 16 + 1
    packed = np.zeros(words, np.uint32)
    offsets = np.zeros(len(enc) + 1, np.uint64)
    kept = _lib.c_u64()
    skipped = _lib.c_u64()
    _lib.call("gdbg_pack_reads", data, _p(so, _lib.u64p), len(enc), min_length,
              _p(packed, _lib.u32p), words, _p(offsets, _lib.u64p), kept, skipped)
    n = int(kept.value)
    used = (int(offsets[n]) + 15) // 16
    return PackedReads(packed[:max(used, 1)].copy(), offsets[:n + 1].copy(), int(skipped.value))


def pack_codes(codes):
    """uint8 codes (A=0 C=1 G=2 T=3) -> uint32 packed stream."""
    codes = np.ascontiguousarray(codes, np.uint8)
    packed = np.zeros(len(codes) // 16 + 1, np.uint32)
    _lib.call("gdbg_pack_codes", _p(codes, _lib.u8p), len(codes), _p(packed, _lib.u32p))
    return packed


def from_codes(reads):
    """List / 2-D array of code rows -> PackedReads (no filtering)."""
    if isinstance(reads, np.ndarray) and reads.ndim == 2:
        flat = np.ascontiguousarray(reads, np.uint8).reshape(-1)
        L = reads.shape[1]
        offsets = np.arange(reads.shape[0] + 1, dtype=np.uint64) * np.uint64(L)
    else:
        rows = [np.asarray(r, np.uint8) for r in reads]
        flat = np.concatenate(rows) if rows else np.zeros(0, np.uint8)
        offsets = np.zeros(len(rows) + 1, np.uint64)
        if rows:
            offsets[1:] = np.cumsum([len(r) for r in rows], dtype=np.uint64)
    return PackedReads(pack_codes(flat), offsets, 0)


def codes_to_str(codes):
    return "".join("ACGT"[int(c)] for c in codes)


def str_to_codes(s):
    t = {"A": 0, "C": 1, "G": 2, "T": 3}
    return np.array([t[c] for c in s], np.uint8)


def concat(parts):
    """One contiguous PackedReads from several (bases re-aligned by shifting
    each part's words to where the previous part ended)."""
    total = sum(int(p.offsets[-1]) for p in parts)
    out = np.zeros(total // 16 + 2, np.uint64)
    offs = [np.zeros(1, np.uint64)]
    B = 0
    for p in parts:
        nb = int(p.offsets[-1])
        nw = (nb + 15) // 16
        if nw:
            words = p.packed[:nw].astype(np.uint64)
            if nb % 16:   # clear bits past the part's last base
                words[-1] &= np.uint64((1 << (2 * (nb % 16))) - 1)
            w, sh = B // 16, 2 * (B % 16)
            out[w:w + nw] |= (words << np.uint64(sh)) & np.uint64(0xFFFFFFFF)
            if sh:
                out[w + 1:w + 1 + nw] |= words >> np.uint64(32 - sh)
        offs.append(p.offsets[1:].astype(np.uint64) + np.uint64(B))
        B += nb
    return PackedReads(out.astype(np.uint32), np.concatenate(offs))


def parse_fastx_device(text, min_length=0, stream=None):
    """FASTA / FASTQ text (torch uint8 CUDA tensor) -> what FastxParser's
    next() yields, packed on the GPU (gdbg_parse_fastx_device).  Returns
    (packed int32 tensor, offsets int64 tensor of n_kept+1, stats dict with
    n_kept / n_dropped / n_parsed / n_skipped).  Text outside the regular
    FASTA / four-line FASTQ layouts raises GoetiaError with code
    ERR_UNSUPPORTED: parse it on the host."""
    import torch
    if text.dtype != torch.uint8 or not text.is_cuda or not text.is_contiguous():
        raise ValueError("parse_fastx_device: text must be a contiguous uint8 CUDA tensor")
    dev = text.device
    n = int(text.numel())
    words = n // 16 + 1
    packed = torch.empty(words, dtype=torch.int32, device=dev)
    # a guess of one record per 32 bytes; a text of shorter records is parsed
    # again with the record count the first call reports
    cap = n // 32 + 2
    st = np.zeros(4, np.uint64)
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        offsets = torch.empty(cap, dtype=torch.int64, device=dev)
        rc = _lib.load().gdbg_parse_fastx_device(text.data_ptr() if n else None, n, min_length,
                                                 packed.data_ptr(), words, offsets.data_ptr(), cap,
                                                 _p(st, _lib.u64p), stream or None)
        if rc == _lib.ERR_INVALID_ARG and int(st[2]) + 1 > cap:
            cap = int(st[2]) + 1
            continue
        _lib.check(rc)
        break
    k = int(st[0])
    return packed, offsets[:k + 1], {"n_kept": k, "n_dropped": int(st[1]),
                                     "n_parsed": int(st[2]), "n_skipped": int(st[3])}


def pack_reads_device(seqs, seq_offsets, min_length=0, stream=None):
    """pack_reads on the GPU.  seqs: torch uint8 CUDA tensor of the reads'
    bytes; seq_offsets: torch int64 CUDA tensor of n+1 byte offsets.
    Returns (packed int32 tensor, offsets int64 tensor of n_kept+1, n_kept,
    n_skipped), all on the same device."""
    import torch
    n = int(seq_offsets.numel()) - 1
    dev = seqs.device
    words = int(seqs.numel()) // 16 + 1
    packed = torch.empty(words, dtype=torch.int32, device=dev)
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    kept, skipped = _lib.c_u64(), _lib.c_u64()
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.call("gdbg_pack_reads_device", seqs.data_ptr(), seq_offsets.data_ptr(), n, min_length,
              packed.data_ptr(), words, offsets.data_ptr(), kept, skipped, stream or None)
    k = int(kept.value)
    return packed, offsets[:k + 1], k, int(skipped.value)
