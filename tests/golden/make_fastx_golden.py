"""Generate tests/golden/fastx.npz from the reference's own FASTX parser.

Runs oracle/_ref/ref_fastx (goetia's FastxParser<DNA_SIMPLE> over its
vendored kseq.h, compiled from the reference sources by
``make -C oracle ref-fastx``) on seeded FASTA / FASTQ texts and stores, per
case and min_length, the sequences next() returned, n_parsed, n_skipped and
whether next() threw InvalidRead.  The texts cover the regular layouts the
GPU parser takes (four-line FASTQ records; FASTA with sequences over any
number of lines, '>' or '@' headers, blank lines) with lower case, 'N' and
other symbols, CRLF line ends, empty sequences, a last line without a
newline and a lone '\\r' ending the text, and layouts it refuses (quality
over several lines, junk before the first header, trailing blank lines
after a FASTQ record, a '+' line in FASTA, a line holding only '\\r' under
a header, a one-byte header at the end, a quality line longer than its
sequence).

    GOETIA_REF=<goetia checkout> python tests/golden/make_fastx_golden.py

Needs the reference checkout, so it runs in the build container only; the
fixture it writes is committed and is all the tests read.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_fastx")
MIN_LENGTHS = (0, 50)


def _seq(rng, n, lower=0.0, other=0.0):
    s = rng.choice(list(b"ACGT"), n).astype(np.uint8)
    if lower:
        m = rng.random(n) < lower
        s[m] = s[m] | 0x20
    if other:
        m = rng.random(n) < other
        s[m] = rng.choice(list(b"NnRY.-*"), int(m.sum()))
    return bytes(s)


def fastq_regular(rng, n_reads, crlf_frac=0.0, max_len=180):
    out = []
    for i in range(n_reads):
        L = int(rng.integers(0, max_len + 1)) if i % 17 else 0
        s = _seq(rng, L, lower=0.05 if i % 3 == 0 else 0.0, other=0.004 if i % 5 == 0 else 0.0)
        q = bytes(rng.integers(33, 75, L).astype(np.uint8))
        q = q.replace(b"@", b"I")[:L] if i % 2 else q   # quality may start with '@' too
        nl = b"\r\n" if rng.random() < crlf_frac else b"\n"
        head = b"@read%d" % i + (b" comment %d" % i if i % 4 == 0 else b"")
        out.append(head + nl + s + nl + b"+" + (b"read%d" % i if i % 6 == 0 else b"") + nl + q + nl)
    text = b"".join(out)
    return text.rstrip(b"\n").rstrip(b"\r") if n_reads % 2 else text   # no final newline


def fasta_multiline(rng, n_reads, crlf_frac=0.0, width=60):
    out = []
    for i in range(n_reads):
        L = int(rng.integers(0, 400)) if i % 11 else 0
        s = _seq(rng, L, lower=0.05 if i % 3 == 0 else 0.0, other=0.003 if i % 4 == 0 else 0.0)
        nl = b"\r\n" if rng.random() < crlf_frac else b"\n"
        head = (b"@" if i % 7 == 3 else b">") + b"seq%d" % i + (b"\tdesc" if i % 5 == 0 else b"")
        lines = [s[j:j + width] for j in range(0, len(s), width)]
        if i % 9 == 4 and lines:
            lines.insert(len(lines) // 2, b"")   # a blank line inside the sequence
        out.append(head + nl + b"".join(x + nl for x in lines))
    return b"".join(out)


def cases():
    rng = np.random.default_rng(20)
    c = {}
    c["fq_regular"] = fastq_regular(rng, 301)
    c["fq_crlf"] = fastq_regular(rng, 120, crlf_frac=1.0)
    c["fq_mixed_eol"] = fastq_regular(rng, 150, crlf_frac=0.3)
    c["fq_short_reads"] = fastq_regular(rng, 200, max_len=60)
    c["fa_multiline"] = fasta_multiline(rng, 160)
    c["fa_crlf"] = fasta_multiline(rng, 80, crlf_frac=0.5)
    c["fa_single_line"] = fasta_multiline(rng, 120, width=1 << 20)
    c["empty"] = b""
    c["fa_header_only_eof"] = b">a\nACGT\n>b desc"
    c["fq_cr_only_seq"] = b"@a\n\r\n+\n\r\n@b\nACGT\n+\nIIII\n"
    # a lone '\r' that ends the text stays in the sequence (its line read
    # meets the end first); one under a sequence line elsewhere is dropped
    c["fa_cr_at_end"] = b">a\nACGT\n\r\nGG\n>b\nACGT\r\n\r"
    c["fa_cr_at_end_after_header"] = b">a\nACGT\n>b\n\r"
    # layouts the GPU parser refuses
    c["x_fq_multiline_qual"] = b"@a\nACGTACGT\n+\nIIII\nIIII\n@b\nAC\n+\nII\n"
    c["x_fq_multiline_seq"] = b"@a\nACGT\nACGT\n+\nIIIIIIII\n"
    c["x_fq_qual_longer"] = b"@a\nACGT\n+\nIIII\n@b\nACGT\n+\nIIIII\n@c\nAC\n+\nII\n"
    c["x_fq_qual_shorter"] = b"@a\nACGT\n+\nII\n@b\nAC\n+\nII\n"
    c["x_junk_prefix"] = b"junk line\n>a\nACGT\n>b\nGG\n"
    c["x_fq_trailing_blank"] = fastq_regular(rng, 10) + b"\n\n"
    c["x_fa_plus_line"] = b">a\nACGT\n+x\nACGT\n>b\nAC\n"
    c["x_fa_cr_only_line"] = b">a\nACGT\n\r\nACGT\n>b\n\r\nAC\n"
    c["x_header_char_at_eof"] = b">a\nACGT\n>"
    c["x_newline_first"] = b"\n>a\nACGT\n"
    return c


def run_ref(paths, min_length):
    out = subprocess.run([DRIVER, str(min_length)] + paths, check=True, capture_output=True).stdout
    res, cur = {}, None
    for line in out.split(b"\n"):
        if line.startswith(b"F "):
            cur = {"seqs": [], "invalid": False}
            res[line[2:].decode()] = cur
        elif line.startswith(b"S "):
            cur["seqs"].append(line[2:])
        elif line.startswith(b"P "):
            f = line.split()
            cur["n_parsed"], cur["n_skipped"] = int(f[1]), int(f[3])
        elif line == b"E":
            cur["invalid"] = True
    return res


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference parser first: make -C oracle ref-fastx REF=<goetia checkout>")
    cs = cases()
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        paths = {}
        for name, text in cs.items():
            p = os.path.join(tmp, name + ".fx")
            with open(p, "wb") as f:
                f.write(text)
            paths[name] = p
        for ml in MIN_LENGTHS:
            res = run_ref(list(paths.values()), ml)
            for name in cs:
                r = res[paths[name]]
                key = f"{name}__m{ml}"
                seqs = r["seqs"]
                off = np.zeros(len(seqs) + 1, np.uint64)
                off[1:] = np.cumsum([len(s) for s in seqs])
                arrays[key + "__seq"] = np.frombuffer(b"".join(seqs), np.uint8)
                arrays[key + "__off"] = off
                arrays[key + "__stats"] = np.array([r["n_parsed"], r["n_skipped"],
                                                    int(r["invalid"])], np.int64)
    for name, text in cs.items():
        arrays[name + "__text"] = np.frombuffer(text, np.uint8)
    arrays["names"] = np.array(list(cs.keys()))
    arrays["min_lengths"] = np.array(MIN_LENGTHS, np.int64)
    np.savez_compressed(os.path.join(HERE, "fastx.npz"), **arrays)
    print("wrote", os.path.join(HERE, "fastx.npz"), len(cs), "cases")


if __name__ == "__main__":
    main()
