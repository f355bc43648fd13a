"""gzip row output (no GPU): blocks deflated in parallel into gzip members
read back as one stream by Python's gzip (as by gunzip / zcat)."""
import gzip
import random

import pytest


def rows(n, seed):
    rng = random.Random(seed)
    out = []
    for i in range(n):
        dna = "".join(rng.choice("ACGTacgt") for _ in range(23))
        out.append(f"{i % 7}\tX\tGGCCGACCTGTCGCTGACGCNNN\t{dna}\tchr{i % 24}\t{rng.randrange(10**8)}\t+\t3\t0\n")
    return "".join(out).encode()


@pytest.mark.parametrize("threads,level", [(1, 1), (4, 1), (0, 6)])
def test_members_read_back_as_one_stream(P, built, tmp_path, threads, level):
    data = rows(250_000, threads)  # ~20 MB: three 8 MiB blocks
    assert len(data) > 2 * (8 << 20)
    path = str(tmp_path / "out.tsv.gz")
    # uneven writes, some straddling block boundaries
    rng = random.Random(1)
    parts, at = [], 0
    while at < len(data):
        n = rng.choice([1, 100, 65536, 3 << 20, 9 << 20])
        parts.append(data[at:at + n])
        at += n
    P.gzip_write(path, parts, level=level, threads=threads)
    raw = open(path, "rb").read()
    assert raw[:2] == b"\x1f\x8b"
    assert len(raw) < len(data) // 2
    assert gzip.decompress(raw) == data


def test_empty_output(P, built, tmp_path):
    path = str(tmp_path / "empty.gz")
    P.gzip_write(path, [])
    assert gzip.decompress(open(path, "rb").read()) == b""
    P.gzip_write(path, [b"", b"x"])
    assert gzip.decompress(open(path, "rb").read()) == b"x"
