"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_driver (goetia's own C++ hot path, compiled from the
reference sources by ``make -C oracle ref``) on seeded read sets and stores
its answers: k-mer hashes, per-read new-k-mer counts, table bytes,
query_sequence counts, neighbour masks, find_decision_kmers positions,
n_unique / n_occupied, the OXLI file written by dBG::save, the
insert_and_query_sequence counts, the compactor's per-k-mer new / seen flags
and neighbour masks with the read's new k-mers (second half of the reads
against a graph of the first half) and (Bit) the
tables after BitStorage::update_from of two half-read graphs.  The cases cover every storage kind, both shifters,
K = 21, 27, 31, 64 (rotation by K mod 64 == 0) and 101 (K > 64), short
reads, duplicate reads, reverse-complement reads, tiny tables (collisions)
and homopolymers (Byte saturation at 255, Nibble at 15).

    GOETIA_REF=<goetia checkout> python tests/golden/make_golden.py

Needs the reference checkout, so it runs in the build container only; the
fixtures it writes are committed and are all the tests read.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name, storage, shifter, K, n_tables, max_table, n_reads, read_len, genome_len, seed
CASES = [
    ("bit_can_k31", "bit", "can", 31, 4, 20000, 60, 150, 3000, 11),
    ("bit_can_k31_tiny", "bit", "can", 31, 4, 211, 40, 120, 2000, 12),
    ("bit_fwd_k27", "bit", "fwd", 27, 3, 5000, 40, 100, 2000, 13),
    ("byte_can_k31", "byte", "can", 31, 4, 4000, 50, 150, 2500, 14),
    ("byte_fwd_k101", "byte", "fwd", 101, 2, 3000, 20, 180, 1500, 15),
    ("nibble_fwd_k21", "nibble", "fwd", 21, 4, 3001, 50, 150, 2500, 16),
    ("nibble_can_k64", "nibble", "can", 64, 4, 5000, 30, 140, 2000, 17),
    ("bit_can_k21_n1", "bit", "can", 21, 1, 1000, 30, 80, 1500, 18),
]


def make_reads(K, n_reads, L, glen, seed):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 4, glen, dtype=np.uint8)
    reads = []
    for _ in range(n_reads):
        s = int(rng.integers(0, glen - L + 1))
        r = g[s:s + L].copy()
        if rng.random() < 0.5:
            r = (3 - r[::-1]).astype(np.uint8)
        m = rng.random(L) < 0.01
        r[m] = (r[m] + rng.integers(1, 4, int(m.sum()), dtype=np.uint8)) & 3
        reads.append("".join("ACGT"[c] for c in r))
    # edge cases: duplicate read, short read, length-K read, homopolymers
    reads.insert(3, reads[1])
    reads.insert(5, reads[2][:max(K - 1, 1)])
    reads.insert(7, reads[4][:K])
    reads.append("")
    reads += ["A" * max(L, K + 40)] * 3
    reads += ["AC" * ((K + 30) // 2 + 1)] * 2
    reads.append(reads[0])
    return reads


def run_case(case, workdir):
    name, kind, shifter, K, N, max_table, n_reads, L, glen, seed = case
    reads = make_reads(K, n_reads, L, glen, seed)
    rfile = os.path.join(workdir, name + ".txt")
    with open(rfile, "w") as f:
        f.write("\n".join(reads) + "\n")
    out = os.path.join(workdir, name)
    os.makedirs(out, exist_ok=True)
    subprocess.check_call([DRIVER, kind, shifter, str(K), str(N), str(max_table), rfile, out])

    def rd(f, dt):
        return np.fromfile(os.path.join(out, f), dt)

    sizes = rd("sizes.u64", np.uint64)
    data = {
        "storage": np.array(kind), "shifter": np.array(shifter), "K": np.array(K),
        "n_tables": np.array(N), "max_table": np.array(max_table),
        "seq": np.frombuffer("".join(reads).encode(), np.uint8),
        "seq_off": np.concatenate([[0], np.cumsum([len(r) for r in reads])]).astype(np.uint64),
        "sizes": sizes,
        "n_new": rd("n_new.u64", np.uint64), "n_kmers": rd("n_kmers.u64", np.uint64),
        "val": rd("val.u64", np.uint64),
        "counts": rd("counts.i16", np.int16), "masks": rd("masks.u8", np.uint8),
        "dpos_read": rd("dpos_read.u64", np.uint64), "dpos_pos": rd("dpos_pos.u64", np.uint64),
        "stats": rd("stats.u64", np.uint64),
    }
    if shifter == "can":
        data["fw"] = rd("fw.u64", np.uint64)
        data["rc"] = rd("rc.u64", np.uint64)
    tables = [rd(f"table{i}.u8", np.uint8) for i in range(len(sizes))]
    data["tables"] = np.concatenate(tables)
    data["table_bytes"] = np.array([len(t) for t in tables], np.uint64)
    data["oxli"] = rd("saved.oxli", np.uint8)
    data["iq_counts"] = rd("iq_counts.i16", np.int16)
    data["compactor_flags"] = rd("compactor_flags.u8", np.uint8)
    data["compactor_masks"] = rd("compactor_masks.u8", np.uint8)
    if kind == "bit":
        data["merge_stats"] = rd("merge_stats.u64", np.uint64)
        data["merged"] = rd("merged.u8", np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
    return name, len(data["val"])


def main():
    if not os.path.exists(DRIVER):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j8"])
    with tempfile.TemporaryDirectory() as td:
        for case in CASES:
            name, nk = run_case(case, td)
            print(f"{name}: {nk} k-mers")


if __name__ == "__main__":
    sys.exit(main())
