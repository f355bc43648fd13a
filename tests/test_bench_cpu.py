"""Host logic of bench.py's workload on CPU: the CPU samples (the reference
arm's and the CPU baseline's) are the leading bytes of the same synthetic
genome the GPU arm searches."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_genome_prefix_is_the_whole_genomes_prefix(P, built):
    sys.path.insert(0, ROOT)
    import bench
    total = 0.2e9  # 24 records of 2-10 Mbp: the prefix spans more than one record
    whole, names, starts, lens = bench.build_genome(P, total)
    for sample in (1_000_000, lens[0] + 1 + lens[1] // 2):
        part, pnames, pstarts, plens = bench.build_genome(P, total, prefix_bp=sample)
        assert len(part) >= sample
        assert bytes(part[:sample]) == bytes(whole[:sample])
        assert pnames == names[:len(pnames)] and pstarts == starts[:len(pstarts)]
        assert plens == lens[:len(plens)]
    # N runs are placed over a record's full length: the prefix holds some.
    assert b"N" in bytes(whole[:lens[0]])


def test_standalone_writer_matches_the_library(P, built, tmp_path):
    """cof-synth (the writer the CPU arms and the verification use, loading
    no library) writes exactly the genome the GPU arm packs: the same record
    lengths, a cut prefix as FASTA, and leading records as 2BIT, as the
    engine's loaders read them back."""
    sys.path.insert(0, ROOT)
    import bench
    total = 0.2e9
    whole, names, starts, lens = bench.build_genome(P, total)
    assert lens == bench.genome_lengths(total)
    limit = lens[0] + 1 + lens[1] // 2
    fa = bench.write_genome(str(tmp_path / "p.fa"), lens, limit=limit)
    assert P.genome_text(fa) == bytes(whole[:limit])
    tb = bench.write_genome(str(tmp_path / "g.2bit"), lens, records=3)
    assert P.genome_text(tb) == bytes(whole[:sum(lens[:3]) + 2])


def test_row_filter_and_comparison():
    sys.path.insert(0, ROOT)
    import bench
    rows = (b"##h\n#c\n0\tX\tA\tA\tchr1\t5\t+\t0\t0\n0\tX\tA\tA\tchr2\t5\t+\t0\t0\n"
            b"1\tX\tA\tA\tchr1\t9\t-\t1\t0\n")
    kept = bench.rows_of_records(rows, ["chr1"])
    assert kept == b"0\tX\tA\tA\tchr1\t5\t+\t0\t0\n1\tX\tA\tA\tchr1\t9\t-\t1\t0\n"
    assert bench.compare_rows(kept, kept)["identical"]
    c = bench.compare_rows(kept, kept.replace(b"\t9\t", b"\t8\t"))
    assert not c["identical"] and c["first_difference"]["row"] == 1
    assert c["rows_compared"] == 2
