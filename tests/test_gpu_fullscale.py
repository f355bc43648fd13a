"""Full-scale plain search (the 3.1 Gbp synthetic genome of 24 records, NRG
with DNA bulge 2 and RNA bulge 1, 4 guides, mm 5):

- whole-genome parity: every row of the GPU search, over all 24 records and
  all 47 segments of 2^26 start positions (so every segment boundary), is
  byte for byte the oracle's row, in the same order, the oracle searching
  the same genome written as 2BIT by the standalone writer;
- every sampled row is consistent with the genome: its DNA column is a
  window at the reported location and strand, lower case exactly where the
  IUPAC rule says mismatch against an aligned crRNA letter, and the number of
  lower-case letters equals the mismatch column (at most the guide's limit;
  at most the column for '-' strand RNA-bulge rows, whose shown window is
  cut short).  The same checks hold on every row of the golden fixtures."""
import os
import random
import sys

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMP = bytes.maketrans(b"ACGTRYKMBVDHacgtrykmbvdh", b"TGCAYRMKVBHDtgcayrmkvbhd")


@pytest.fixture(scope="module")
def full(P, built):
    sys.path.insert(0, ROOT)
    import bench
    buf, names, starts, lens = bench.build_genome(P, 3.1e9)
    n = len(buf)
    W = P.plane_words(n)
    planes = np.empty(3 * W, dtype=np.uint32)
    hi, lo, ot = planes[:W], planes[W:2 * W], planes[2 * W:]
    P.pack_text(buf, out=(hi, lo, ot))
    guides = bench.make_guides()
    with P.CasOFFinder(0) as eng:
        eng.readInputFile(bench.input_text("synthetic", guides))
        eng.load_genome_planes(hi, lo, ot, n, None, None, names, starts)
        rows = eng.search()
    return bench, buf, names, starts, guides, rows


def test_whole_genome_rows_equal_the_oracle(full, oracle, tmp_path):
    bench, buf, names, starts, guides, rows = full
    lens = bench.genome_lengths(3.1e9)
    assert [s for s in starts] == [sum(lens[:i]) + i for i in range(len(lens))]
    path = bench.write_genome(str(tmp_path / "genome.2bit"), lens)
    _, want = bench.oracle_rows(oracle, bench.input_text(path, guides), os.cpu_count() or 1, str(tmp_path), "full")
    c = bench.compare_rows(rows, want)
    assert c["rows_compared"] > 1_000_000
    assert c["identical"], c["first_difference"]


def test_sampled_rows_agree_with_the_genome(full):
    bench, buf, names, starts, guides, rows = full
    all_rows = cases.rows_of(rows)
    assert len(all_rows) > 500_000
    rec = {nm: st for nm, st in zip(names, starts)}
    rng = random.Random(8)
    for r in rng.sample(all_rows, 3000):
        f = r.decode().split("\t")
        crrna, dna, chrom, loc, strand, mm = f[2], f[3], f[4], int(f[5]), f[6], int(f[7])
        assert mm <= bench.MM
        bases = [c for c in dna if c != "-"]
        # The DNA column (oriented window, padding and bulge offsets applied
        # by the reference's row rules) lies within a few positions of the
        # reported location on the reported strand.
        g0 = rec[chrom] + loc
        near = bytes(buf[max(0, g0 - 8):g0 + len(bases) + 8])
        if strand == "-":
            near = near.translate(COMP)[::-1]
        assert "".join(bases).upper().encode() in near.upper(), r
        assert not cases.row_problems(r.decode()), r

