"""Batched search: several input files over one resident genome in one pass.

Each job must give exactly the rows the oracle gives for that input file run
alone -- jobs sharing a padded pattern share the PAM scan and the comparer
launch, but never merge compare keys, ids or thresholds across jobs."""
import os
import random

import pytest

import cases

pytestmark = pytest.mark.gpu

NGG = "N" * 21 + "GG"


def batch_inputs(rng, genome):
    """(pattern line, guide lines) per job; jobs 0 and 1 share a pattern."""
    def g(n, spacer, pam_n, pam5=False):
        out = []
        for _ in range(n):
            sp = "".join(rng.choice("ACGT") for _ in range(spacer))
            out.append(("N" * pam_n + sp) if pam5 else (sp + "N" * pam_n))
        return out
    shared = g(2, 20, 3)
    jobs = [
        (NGG + " 1 1", [f"{x} 5" for x in shared]),
        (NGG + " 1 1", [f"{x} 4 dup{i}" for i, x in enumerate(shared + g(1, 20, 3))]),  # same keys, other ids
        ("N" * 21 + "RG 2 1", [f"{x} 5" for x in g(3, 20, 3)]),
        ("TTTV" + "N" * 23 + " 1 1", [f"{x} 4" for x in g(2, 23, 4, pam5=True)]),
        ("N" * 21 + "NNGRRT", [f"{x} 3" for x in g(2, 21, 6)]),
        (NGG, [f"{x} 3" for x in g(1, 20, 3)]),
    ]
    return [f"{genome}\n{p}\n" + "\n".join(gl) + "\n" for p, gl in jobs]


def test_batch_matches_single_job_oracle(P, built, oracle, tmp_path):
    rng = random.Random(77)
    seqs = [P.synth_record(301, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
            for r, n in enumerate([150000, 90000])]
    genome = str(tmp_path / "genome.fa")
    texts = batch_inputs(rng, genome)
    # Plant mutated sites of every job's guides so that each job has hits.
    for t in texts:
        lines = t.strip().split("\n")
        pat = lines[1].split()
        dna = int(pat[1]) if len(pat) == 3 else 0
        rna = int(pat[2]) if len(pat) == 3 else 0
        guides = [l.split()[0] for l in lines[2:]]
        cases.plant_sites(rng, seqs, pat[0], guides, 25, 6, dna, rna)
    P.write_fasta(genome, ["chr1", "chr2"], seqs)
    want, want_summ = [], []
    for j, t in enumerate(texts):
        path = str(tmp_path / f"job{j}.txt")
        open(path, "w").write(t)
        out = str(tmp_path / f"job{j}.tsv")
        summ = str(tmp_path / f"job{j}_summary.txt")
        r = cases.run_cli(oracle, path, out, threads=4, summary=summ)
        assert r.returncode == 0, r.stderr.decode()
        want.append(open(out, "rb").read())
        want_summ.append(open(summ, "rb").read())
        assert len(cases.rows_of(want[-1])) > 0, f"job {j} has no hits"
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        for t in texts:
            eng.batch_add_input(t)
        assert eng.batch_size() == len(texts)
        eng.set_summary(True)
        allrows = eng.search()
        got = [eng.job_rows(j) for j in range(len(texts))]
        assert b"".join(got) == allrows
        for j in range(len(texts)):
            assert P.HEADER.encode() + got[j] == want[j], f"job {j}"
            assert eng.job_summary(j) == want_summ[j], f"job {j} summary"
        # A second search of the same batch gives the same rows.
        assert eng.search() == allrows
        # Single-job API after a batch: replaces the batch.
        eng.readInputFile(texts[2])
        assert P.HEADER.encode() + eng.search() == want[2]


def test_batch_mixed_jobs_and_large_group(P, built, oracle, tmp_path):
    """48 jobs of the 1,024-guide mixed workload's shape (spacer 20-24, NGG/NRG,
    2% IUPAC codes, mm 3-6, DNA bulge 0-2, RNA bulge 0-1) plus one job whose
    pattern group has more than 256 compare variants, each checked against the
    oracle run on that input alone."""
    import bench
    rng = random.Random(91)
    seqs = [P.synth_record(411, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
            for r, n in enumerate([400000, 250000])]
    genome = str(tmp_path / "genome.fa")
    texts = bench.batched_jobs(seed=17, n=48, genome_path=genome)
    big = [f"{''.join(rng.choice('ACGT') for _ in range(20))}NNN 5" for _ in range(6)]
    texts.append(f"{genome}\n{'N' * 21}GG 2 1\n" + "\n".join(big) + "\n")  # 6 x ~57 variants in one group
    for t in texts:
        lines = t.strip().split("\n")
        pat = lines[1].split()
        dna = int(pat[1]) if len(pat) == 3 else 0
        rna = int(pat[2]) if len(pat) == 3 else 0
        cases.plant_sites(rng, seqs, pat[0], [l.split()[0] for l in lines[2:]], 6, 5, dna, rna)
    P.write_fasta(genome, ["chr1", "chr2"], seqs)
    want = []
    for j, t in enumerate(texts):
        path = str(tmp_path / f"job{j}.txt")
        open(path, "w").write(t)
        out = str(tmp_path / f"job{j}.tsv")
        r = cases.run_cli(oracle, path, out, threads=8)
        assert r.returncode == 0, r.stderr.decode()
        want.append(open(out, "rb").read())
    assert sum(len(cases.rows_of(w)) for w in want) > 100
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        for t in texts:
            eng.batch_add_input(t)
        assert eng.input_info()["variants"] > 256 + 48
        eng.search()
        for j in range(len(texts)):
            assert P.HEADER.encode() + eng.job_rows(j) == want[j], f"job {j}"
