"""The oracle (CPU restatement) against the reference's own outputs.

Golden fixtures hold outputs of the reference itself (tests/golden/
make_golden.py); the oracle must reproduce each byte for byte when run with
one thread.  When the reference checkout is present, seeded random cases are
also run through both programs here."""
import os
import random
import subprocess

import pytest

import cases
from conftest import GOLDEN, golden_cases, golden_input


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference_golden(case, oracle, tmp_path):
    d = os.path.join(GOLDEN, case)
    inp = golden_input(case, tmp_path)
    out = str(tmp_path / "out.tsv")
    summ = str(tmp_path / "summary.txt") if os.path.exists(os.path.join(d, "expected_summary.txt")) else None
    r = cases.run_cli(oracle, inp, out, threads=1, summary=summ)
    if os.path.exists(os.path.join(d, "expected_error.txt")):
        code, msg = open(os.path.join(d, "expected_error.txt")).read().split("\n")[:2]
        assert r.returncode == int(code)
        assert msg in r.stderr.decode()
        return
    assert r.returncode == 0, r.stderr.decode()
    assert open(out, "rb").read() == open(os.path.join(d, "expected.tsv"), "rb").read()
    if summ:
        assert open(summ, "rb").read() == open(os.path.join(d, "expected_summary.txt"), "rb").read()


def test_oracle_threads_same_order(oracle, tmp_path):
    inp = golden_input("nrg_bulge_2bit", tmp_path)
    a, b = str(tmp_path / "a.tsv"), str(tmp_path / "b.tsv")
    assert cases.run_cli(oracle, inp, a, threads=1).returncode == 0
    assert cases.run_cli(oracle, inp, b, threads=4).returncode == 0
    assert open(a, "rb").read() == open(b, "rb").read()


RANDOM_CASES = [
    dict(seed=101, lens=[20000, 15000], pattern="N" * 21 + "GG", mm=4),
    dict(seed=102, lens=[30000], fmt="2bit", pattern="N" * 21 + "RG", dna=2, rna=1, mm=5),
    dict(seed=103, lens=[25000, 5000], pattern="TTTN" + "N" * 20, dna=2, rna=2, mm=3),
    dict(seed=104, lens=[20000], pattern="N" * 19 + "NNGRRT", dna=1, rna=0, mm=[2, 6], iupac_frac=0.15,
         sprinkle_chars="RYSWnX"),
    dict(seed=105, lens=[8000, 8000], pattern="N" * 30 + "NGG", dna=1, rna=1, mm=6),
    # The GPU parity cases at the edges of the bit-sliced comparer's narrow
    # counters (tests/test_gpu_parity.py seeds 212 and 213, the same inputs):
    # 20-nt guides at thresholds 4 / 15 and 3 / 16, tens of thousands of rows.
    dict(seed=212, lens=[20000], pattern="N" * 21 + "RG", dna=1, rna=1, mm=[4, 15], per_guide=20,
         guides=["".join(random.Random(212 + i).choice("ACGT") for _ in range(20)) + "NNN" for i in range(2)]),
    dict(seed=213, lens=[20000], pattern="N" * 21 + "RG", dna=1, rna=1, mm=[3, 16], per_guide=20,
         guides=["".join(random.Random(213 + i).choice("ACGT") for _ in range(20)) + "NNN" for i in range(2)]),
    # and its multi-chunk groups (seeds 214, 215): ~700 variants.
    dict(seed=214, lens=[100000], pattern="N" * 21 + "RG", dna=2, rna=1, mm=5, n_guides=12, per_guide=10),
    dict(seed=215, lens=[100000], pattern="N" * 21 + "RG", dna=2, rna=1, mm=[3, 5], n_guides=12, per_guide=10),
]


@pytest.mark.parametrize("spec", RANDOM_CASES, ids=[str(c["seed"]) for c in RANDOM_CASES])
def test_oracle_matches_reference_random(spec, oracle, reference, tmp_path):
    if reference is None:
        pytest.skip("reference checkout not present")
    inp, _ = cases.make_case(str(tmp_path), **spec)
    a, b = str(tmp_path / "ref.tsv"), str(tmp_path / "ora.tsv")
    ra = cases.run_cli(reference, inp, a, threads=1)
    rb = cases.run_cli(oracle, inp, b, threads=1)
    assert ra.returncode == 0 and rb.returncode == 0
    ta, tb = open(a, "rb").read(), open(b, "rb").read()
    assert ta == tb
    assert len(cases.rows_of(ta)) > 0


def test_reference_gpu_kernels_agree(reference, tmp_path):
    """The reference's work-group kernels (finder/comparer, device G) give the
    same rows as its CPU kernels (multiset; atomics reorder them)."""
    if reference is None:
        pytest.skip("reference checkout not present")
    inp = golden_input("nrg_bulge_2bit", tmp_path)
    a, b = str(tmp_path / "c.tsv"), str(tmp_path / "g.tsv")
    assert cases.run_cli(reference, inp, a, threads=2, device="C").returncode == 0
    assert cases.run_cli(reference, inp, b, threads=2, device="G").returncode == 0
    assert cases.canonical(open(a, "rb").read()) == cases.canonical(open(b, "rb").read())


def test_mismatch_predicate_exhaustive(P, built, oracle, tmp_path):
    """All 256 x 256 (pattern byte, genome byte) pairs: the reference kernel's
    predicate (golden table), the oracle's and the engine's class table agree."""
    import numpy as np
    golden = np.fromfile(os.path.join(GOLDEN, "mismatch_table.bin"), np.uint8).reshape(256, 256)
    out = str(tmp_path / "oracle_table.bin")
    assert subprocess.run([oracle, "--mismatch-table", out]).returncode == 0
    ora = np.fromfile(out, np.uint8).reshape(256, 256)
    eng = P.mismatch_table()
    assert (ora == golden).all()
    assert (eng == golden).all()
    assert golden.sum() == 1036  # 4 concrete bases x 255 + 6 two-base codes x 2 + 4 three-base codes x 1


def test_golden_rows_obey_the_row_rules():
    """The genome-free row checks that the full-scale GPU test applies to
    sampled rows hold on every row the reference wrote in the fixtures."""
    n = 0
    for case in golden_cases():
        path = os.path.join(GOLDEN, case, "expected.tsv")
        if not os.path.exists(path):
            continue
        for row in cases.rows_of(open(path, "rb").read()):
            assert not cases.row_problems(row.decode()), (case, row)
            n += 1
    assert n > 4000


def _fasta_records(path):
    names, seqs = [], []
    for line in open(path, "rb").read().split(b"\n"):
        line = line.rstrip(b"\r")
        if line.startswith(b">"):
            names.append(line[1:].decode())
            seqs.append(bytearray())
        elif line:
            seqs[-1] += line.upper()
    return names, seqs


@pytest.mark.parametrize("case", ["ngg_fasta", "iupac_nngrrt"])
def test_kernel_restatement_matches_reference_golden(case, P):
    """cases.restate_finder / restate_comparer (the numpy restatement of
    finder_cpu and comparer_cpu that the chunk-level GPU tests check against)
    give, guide by guide, exactly the hits of the reference's rows on two
    fixtures without bulges, one of them with IUPAC codes in the guides."""
    d = os.path.join(GOLDEN, case)
    lines = open(os.path.join(d, "input.txt")).read().split("\n")
    pattern = lines[1].split()[0].upper().encode()
    names, seqs = _fasta_records(os.path.join(d, "genome.fa"))
    text, starts = P.reference_text(seqs)
    loci, flags = cases.restate_finder(text, pattern)
    rows = cases.rows_of(open(os.path.join(d, "expected.tsv"), "rb").read())
    total = 0
    for no, line in enumerate(l for l in lines[2:] if l.strip()):
        tok = line.split()
        gid = tok[2] if len(tok) == 3 else str(no)
        want = sorted((starts[names.index(r[4].decode())] + int(r[5]), r[6] == b"-", int(r[7]))
                      for r in (x.split(b"\t") for x in rows) if r[0].decode() == gid)
        got = sorted(cases.restate_comparer(text, loci, flags, tok[0].upper().encode(), int(tok[1])))
        assert got == want, gid
        total += len(got)
    assert total == len(rows) > 0
