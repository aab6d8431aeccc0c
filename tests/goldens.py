"""Access to the golden fixtures produced by the reference (tests/golden/)."""
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def names():
    """The dBG cases (fastx.npz holds the FASTX parser cases)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if os.path.basename(p) != "fastx.npz")


class Case:
    def __init__(self, name):
        d = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.name = name
        self.storage = str(d["storage"])
        self.shifter = str(d["shifter"])
        self.canonical = self.shifter == "can"
        self.K = int(d["K"])
        self.sizes = d["sizes"]
        seq, off = d["seq"].tobytes(), d["seq_off"]
        self.reads = [seq[off[i]:off[i + 1]].decode() for i in range(len(off) - 1)]
        self.n_new = d["n_new"]
        self.n_kmers = d["n_kmers"]
        self.val = d["val"]
        self.fw = d["fw"] if "fw" in d else None
        self.rc = d["rc"] if "rc" in d else None
        self.counts = d["counts"]
        self.masks = d["masks"]
        self.dpos = list(zip(d["dpos_read"].tolist(), d["dpos_pos"].tolist()))
        self.n_unique, self.n_occupied = (int(x) for x in d["stats"])
        tb = d["table_bytes"].astype(np.int64)
        t = d["tables"]
        self.tables = [t[a:b] for a, b in zip(np.r_[0, np.cumsum(tb)[:-1]], np.cumsum(tb))]
        self.oxli = d["oxli"].tobytes()     # the file dBG::save wrote
        self.iq_counts = d["iq_counts"]      # insert_and_query_sequence, fresh tables
        # compactor query of the second half of the reads against a graph of the first half
        self.compactor_flags = d["compactor_flags"]
        self.compactor_masks = d["compactor_masks"]
        # Bit only: A (first half of the reads) after A.update_from(B)
        self.merge_stats = d["merge_stats"] if "merge_stats" in d else None
        if "merged" in d:
            self.merged = [d["merged"][a:b] for a, b in
                           zip(np.r_[0, np.cumsum(tb)[:-1]], np.cumsum(tb))]

    def packed(self):
        """2-bit packed batch of the reads (all of them are pure ACGT)."""
        codes = {"A": 0, "C": 1, "G": 2, "T": 3}
        flat = np.array([codes[c] for r in self.reads for c in r], np.uint8)
        off = np.zeros(len(self.reads) + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in self.reads])
        n = len(flat)
        pad = np.zeros((n + 15) // 16 * 16 + 16, np.uint8)
        pad[:n] = flat
        words = (pad.reshape(-1, 16).astype(np.uint32) << (2 * np.arange(16, dtype=np.uint32))).sum(1)
        return words.astype(np.uint32), off

    def decision_positions(self, masks):
        """(read, pos) of k-mers whose mask has >1 left or >1 right neighbour."""
        out, k = [], 0
        for r, s in enumerate(self.reads):
            n = max(len(s) - self.K + 1, 0)
            for p in range(n):
                m = int(masks[k + p])
                if bin(m & 15).count("1") > 1 or bin(m >> 4).count("1") > 1:
                    out.append((r, p))
            k += n
        return out
