"""Speed of the C restatement (goetia_oracle.c) against the reference's own
insert path on this host: one thread each, the same seeded reads, the same
table sizes, dBG<ByteStorage, CanLemireShifter> with K=31 and 4 tables.  It
checks that the restatement, which the benchmark's reference arm times
because the reference's objects do not travel to other hosts, is a fair
stand-in for the reference's code.  Test infrastructure: needs the reference
build (make -C oracle ref) and prints one line per table size.

    python oracle/port_speed.py [n_reads]
"""
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle  # noqa: E402

DRIVER = os.path.join(HERE, "_ref", "ref_driver")
K = 31


def seeded_reads(n_reads, read_len=150, genome_bp=50_000_000, sub_rate=0.005, seed=3):
    rng = np.random.default_rng(seed)
    genome = rng.integers(0, 4, genome_bp, dtype=np.uint8)
    starts = rng.integers(0, genome_bp - read_len, n_reads)
    rows = genome[starts[:, None] + np.arange(read_len)]
    hit = rng.random(rows.shape) < sub_rate
    rows[hit] = (rows[hit] + rng.integers(1, 4, int(hit.sum()), dtype=np.uint8)) % 4
    return rows


def packed_of(rows):
    codes = rows.reshape(-1).astype(np.uint32)
    idx = np.arange(len(codes), dtype=np.uint64)
    packed = np.zeros(len(codes) // 16 + 1, np.uint32)
    np.bitwise_or.at(packed, idx >> 4, codes << (2 * (idx & 15)).astype(np.uint32))
    offsets = np.arange(rows.shape[0] + 1, dtype=np.uint64) * np.uint64(rows.shape[1])
    return packed, offsets


def main():
    n_reads = int(sys.argv[1]) if len(sys.argv) > 1 else 200_000
    if not os.path.exists(DRIVER):
        sys.exit(f"{DRIVER} is missing: run `make -C oracle ref` first")
    rows = seeded_reads(n_reads)
    packed, offsets = packed_of(rows)
    letters = np.frombuffer(b"ACGT", np.uint8)[rows]
    with tempfile.NamedTemporaryFile("wb", suffix=".txt", delete=False) as f:
        f.write(b"\n".join(bytes(r) for r in letters) + b"\n")
        path = f.name
    try:
        for max_table in (1 << 28, 1 << 30):
            out = subprocess.run([DRIVER, "time", "byte", "can", str(K), "4", str(max_table), path],
                                 check=True, capture_output=True, text=True).stdout.split()
            ref_kmers, ref_new, ref_s = int(out[0]), int(out[1]), float(out[2])
            st = oracle.Storage("byte", oracle.primes(4, max_table))
            t0 = time.perf_counter()
            total, n_new = st.insert_reads(True, K, packed, offsets)
            port_s = time.perf_counter() - t0
            assert total == ref_kmers and int(n_new.sum()) == ref_new
            print(f"4 x ~2^{max_table.bit_length() - 1} Byte cells, {n_reads} reads: "
                  f"reference {ref_kmers / ref_s / 1e6:.2f} M k-mers/s, "
                  f"restatement {total / port_s / 1e6:.2f} M k-mers/s "
                  f"(restatement / reference {ref_s / port_s:.2f}), same k-mer and new counts")
    finally:
        os.unlink(path)


if __name__ == "__main__":
    main()
