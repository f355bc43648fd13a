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
