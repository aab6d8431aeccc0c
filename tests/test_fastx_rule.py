"""The per-line rule of the GPU FASTX parser (goetia_gb300/csrc/gdbg_fastx_device.cu),
restated in Python and checked on the CPU against kseq.

The GPU parser finds records line by line and accepts only the layouts where
that gives kseq's answer, declining the rest.  Here the same rule runs on
the reference's FASTX fixtures (tests/golden/fastx.npz: it must reproduce
what the reference's FastxParser returned on every case it accepts, and
decline the cases marked "x_") and on seeded random texts built from FASTA /
FASTQ line kinds (headers, sequence, '+', quality, blank and lone-'\\r'
lines, CRLF ends, junk): whenever the rule accepts a text, its reads,
n_parsed and n_skipped must equal the oracle's kseq restatement, which the
fixtures pin to the reference.  CPU only.
"""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def per_line_rule(text, min_length):
    """(kept reads, n_parsed, n_skipped), or None where the GPU parser declines."""
    n = len(text)
    if n == 0:
        return [], 0, 0
    if text[0] not in b">@":
        return None
    nl = [i for i, c in enumerate(text) if c == 10]
    n_nl = len(nl)
    n_lines = n_nl + (1 if text[-1] != 10 else 0)

    def line(j):
        return (0 if j == 0 else nl[j - 1] + 1), (nl[j] if j < n_nl else n)

    def eff(s, e):
        return e - s - (1 if e - s >= 2 and text[e - 1] == 13 else 0)

    fastq = False
    if text[0] == ord("@") and n_lines >= 3:
        s2, e2 = line(2)
        fastq = e2 > s2 and text[s2] == ord("+")
    recs = []
    for j in range(n_lines):
        s, e = line(j)
        c0 = text[s] if e > s else -1
        if fastq:
            if n_lines % 4:
                return None
            role = j % 4
            if role == 0:
                if c0 != ord("@"):
                    return None
                recs.append(b"")
            elif role == 1:
                if c0 in (ord(">"), ord("+"), ord("@")):
                    return None
                recs[-1] = text[s:s + eff(s, e)]
            elif role == 2:
                if c0 != ord("+"):
                    return None
            elif eff(s, e) != eff(*line(j - 2)):
                return None
        else:
            header = c0 in (ord(">"), ord("@"))
            if c0 == ord("+") or (header and e - s == 1 and j >= n_nl):
                return None
            if e - s == 1 and c0 == 13 and j < n_nl:
                ps, pe = line(j - 1)
                p0 = text[ps] if pe > ps else -1
                if pe == ps or p0 in (ord(">"), ord("@")) or (pe - ps == 1 and p0 == 13):
                    return None
                continue
            if header:
                recs.append(b"")
            else:
                recs[-1] += text[s:s + eff(s, e)]
    kept, skipped = [], 0
    for r in recs:
        valid = all(c in b"ACGTacgt" for c in r)
        short = len(r) < min_length
        skipped += int(not valid) + int(short)
        if valid and not short:
            kept.append(r.upper())
    return kept, len(recs), skipped


def test_rule_on_reference_fixtures():
    z = np.load(os.path.join(HERE, "golden", "fastx.npz"))
    for name in z["names"]:
        text = z[name + "__text"].tobytes()
        for ml in z["min_lengths"]:
            k = f"{name}__m{ml}"
            got = per_line_rule(text, int(ml))
            if name.startswith("x_"):
                assert got is None, k
                continue
            seq, off, st = z[k + "__seq"].tobytes(), z[k + "__off"], z[k + "__stats"]
            gold = [seq[int(off[i]):int(off[i + 1])] for i in range(len(off) - 1)]
            assert got == (gold, int(st[0]), int(st[1])), k


LINE_KINDS = [b">h", b"@h x", b"+", b"+h", b"", b"\r", b"ACGT", b"acgtN", b"GATTACA", b"II",
              b"IIII", b"@@@@", b">", b"@", b"TTTTTTT", b"junk"]


def random_text(rng):
    kinds = rng.integers(0, len(LINE_KINDS), int(rng.integers(1, 14)))
    lines = [LINE_KINDS[k] for k in kinds]
    if rng.random() < 0.5:   # a regular FASTQ record or two now and then
        for _ in range(int(rng.integers(1, 3))):
            L = int(rng.integers(0, 6))
            lines += [b"@r", bytes(rng.choice(list(b"ACGTN"), L)), b"+", b"I" * L]
    eol = b"\r\n" if rng.random() < 0.3 else b"\n"
    text = eol.join(lines)
    return text + eol if rng.random() < 0.6 else text


@pytest.mark.parametrize("seed", range(4))
def test_rule_agrees_with_kseq_when_it_accepts(seed):
    rng = np.random.default_rng(100 + seed)
    accepted = 0
    for _ in range(3000):
        text = random_text(rng)
        for ml in (0, 4):
            got = per_line_rule(text, ml)
            if got is None:
                continue
            accepted += 1
            seqs, st, status = oracle.parse_fastx(text, ml)
            assert status == 0, text
            assert got == (seqs, st["n_parsed"], st["n_skipped"]), text
    assert accepted > 200   # the random texts do exercise accepted layouts


def random_fastq(rng):
    """Mostly four-line FASTQ records whose lines carry the bytes kseq
    treats specially ('@', '>', '+', '\\r', blanks) in odd places."""
    lines = []
    for _ in range(int(rng.integers(1, 6))):
        L = int(rng.integers(0, 7))
        seq = rng.choice(list(b"ACGTNacgt\r@>+I"), L,
                         p=[.12, .12, .12, .12, .04, .08, .08, .08, .08, .04, .03, .03, .02, .04])
        qual = rng.choice(list(b"I@+>\r#"), L)
        head = b"@" + rng.choice(list(b"r \t\r@>+"), int(rng.integers(0, 4))).astype(np.uint8).tobytes()
        plus = b"+" + rng.choice(list(b"r \r@"), int(rng.integers(0, 3))).astype(np.uint8).tobytes()
        rec = [head, seq.astype(np.uint8).tobytes(), plus, qual.astype(np.uint8).tobytes()]
        if rng.random() < 0.3:
            k = int(rng.integers(1, 4))
            rec[k] += b"\r"
        lines += rec
    eol = b"\r\n" if rng.random() < 0.2 else b"\n"
    text = eol.join(lines)
    return text + eol if rng.random() < 0.6 else text


@pytest.mark.parametrize("seed", range(2))
def test_rule_agrees_with_kseq_on_fastq(seed):
    rng = np.random.default_rng(200 + seed)
    accepted = 0
    for _ in range(3000):
        text = random_fastq(rng)
        for ml in (0, 3):
            got = per_line_rule(text, ml)
            if got is None:
                continue
            accepted += 1
            seqs, st, status = oracle.parse_fastx(text, ml)
            assert status == 0, text
            assert got == (seqs, st["n_parsed"], st["n_skipped"]), text
    assert accepted > 2000
