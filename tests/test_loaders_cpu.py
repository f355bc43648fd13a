"""Genome loaders on the host (no GPU): FASTA and 2BIT files to the reference's
genome string.

Version 0 2BIT files laid out back to back are what the reference reads
(read_twobit.cpp:44-131); the loader also honours the index offsets, reads
version 1 (64-bit offsets) and files of the other byte order.  All layouts of
the same records must give the same genome string, the one the FASTA loader
gives for the same sequences."""
import random
import struct

import pytest

TWOBIT = {"T": 0, "C": 1, "A": 2, "G": 3}


def records(seed=4):
    rng = random.Random(seed)
    out = []
    for n in (1000, 37, 2049, 5):
        s = [rng.choice("ACGT") for _ in range(n)]
        for _ in range(3):  # N runs
            a = rng.randrange(n)
            for k in range(a, min(n, a + rng.randint(1, 40))):
                s[k] = "N"
        out.append("".join(s))
    return [f"chr{i}" for i in range(len(out))], out


def record_bytes(seq, endian):
    ns, starts, sizes = False, [], []
    for i, c in enumerate(seq):
        if c == "N" and not ns:
            starts.append(i)
        if c != "N" and ns:
            sizes.append(i - starts[-1])
        ns = c == "N"
    if ns:
        sizes.append(len(seq) - starts[-1])
    codes = [TWOBIT.get(c, 0) for c in seq] + [0] * ((-len(seq)) % 4)
    packed = bytes((codes[i] << 6) | (codes[i + 1] << 4) | (codes[i + 2] << 2) | codes[i + 3]
                   for i in range(0, len(codes), 4))
    b = struct.pack(endian + "II", len(seq), len(starts))
    b += struct.pack(endian + f"{len(starts)}I", *starts) + struct.pack(endian + f"{len(sizes)}I", *sizes)
    b += struct.pack(endian + "II", 0, 0) + packed
    return b


def write_2bit(path, names, seqs, version=0, endian="<", order=None, gap=0):
    """UCSC .2bit with the record data in `order` (index order by default),
    `gap` spare bytes before each record."""
    recs = [record_bytes(s, endian) for s in seqs]
    osz = 8 if version == 1 else 4
    index_size = sum(1 + len(n) + osz for n in names)
    order = order or list(range(len(seqs)))
    offs, at = [0] * len(seqs), 16 + index_size
    for r in order:
        at += gap
        offs[r] = at
        at += len(recs[r])
    out = bytearray(struct.pack(endian + "IIII", 0x1A412743, version, len(names), 0))
    for n, o in zip(names, offs):
        out += bytes([len(n)]) + n.encode() + struct.pack(endian + ("Q" if version == 1 else "I"), o)
    body = bytearray()
    for r in order:
        body += b"\0" * gap + recs[r]
    out += body
    with open(path, "wb") as f:
        f.write(out)


@pytest.fixture(scope="module")
def expected(P):
    names, seqs = records()
    return names, seqs, ";".join(seqs).encode()


def test_fasta_and_back_to_back_2bit_agree(P, tmp_path, expected):
    names, seqs, want = expected
    fa = tmp_path / "g.fa"
    P.write_fasta(str(fa), names, [s.encode() for s in seqs])
    assert P.genome_text(str(fa)) == want
    tb = tmp_path / "g.2bit"
    write_2bit(str(tb), names, seqs)
    assert P.genome_text(str(tb)) == want


@pytest.mark.parametrize("layout", [
    dict(version=1),
    dict(endian=">"),
    dict(version=1, endian=">"),
    dict(order=[2, 0, 3, 1]),
    dict(order=[3, 2, 1, 0], gap=13, version=1),
])
def test_2bit_layouts_beyond_the_reference(P, tmp_path, expected, layout):
    names, seqs, want = expected
    path = tmp_path / "g.2bit"
    write_2bit(str(path), names, seqs, **layout)
    assert P.genome_text(str(path)) == want


def test_back_to_back_2bit_matches_the_oracle(P, built, oracle, tmp_path, expected):
    """The oracle (the reference's reading) on a version 0 file: the same
    genome, seen through a search that reports every candidate site."""
    import cases
    names, seqs, want = expected
    tb = tmp_path / "g.2bit"
    write_2bit(str(tb), names, seqs)
    inp = tmp_path / "in.txt"
    inp.write_text(f"{tb}\n" + "N" * 8 + "GG\n" + "N" * 8 + "NN 0\n")
    out = tmp_path / "out.tsv"
    r = cases.run_cli(oracle, str(inp), str(out), device="C")
    assert r.returncode == 0, r.stderr.decode()
    # every NGG-adjacent window of the genome appears as a row
    rows = [l.split(b"\t") for l in open(out, "rb").read().splitlines() if not l.startswith(b"#")]
    g = want.decode()
    parts = g.split(";")
    for row in rows[:50]:
        chrom, loc, strand = row[4].decode(), int(row[5]), row[6].decode()
        seq = parts[names.index(chrom)]
        win = seq[loc:loc + 10]
        if strand == "+":
            assert win.endswith("GG")
        else:
            assert win.startswith("CC")


def test_not_a_genome(P, tmp_path):
    bad = tmp_path / "x.txt"
    bad.write_text("hello\n")
    assert P.genome_text(str(bad)) is None
    v2 = tmp_path / "v2.2bit"
    with open(v2, "wb") as f:
        f.write(struct.pack("<IIII", 0x1A412743, 2, 0, 0))
    assert P.genome_text(str(v2)) is None
