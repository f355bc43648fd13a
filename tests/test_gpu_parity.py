"""Parity of the GB300 path with the reference (golden fixtures) and the oracle.

All comparisons are byte-exact: the engine emits rows in the order the
reference emits them for one chunk with work-items in order, which is also
the oracle's order."""
import os
import random

import numpy as np
import pytest

import cases
from conftest import GOLDEN, golden_cases, golden_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", golden_cases())
def test_cli_matches_reference_golden(case, P, built, tmp_path):
    d = os.path.join(GOLDEN, case)
    inp = golden_input(case, tmp_path)
    out = str(tmp_path / "out.tsv")
    summ = str(tmp_path / "summary.txt") if os.path.exists(os.path.join(d, "expected_summary.txt")) else None
    r = cases.run_cli(P.CLI_PATH, inp, out, device="G0", summary=summ)
    if os.path.exists(os.path.join(d, "expected_error.txt")):
        code, msg = open(os.path.join(d, "expected_error.txt")).read().split("\n")[:2]
        assert r.returncode == int(code)
        assert msg in r.stderr.decode()
        return
    assert r.returncode == 0, r.stderr.decode()
    got, want = open(out, "rb").read(), open(os.path.join(d, "expected.tsv"), "rb").read()
    if got != want:
        g, w = cases.rows_of(got), cases.rows_of(want)
        extra = sorted(set(g) - set(w))[:5]
        missing = sorted(set(w) - set(g))[:5]
        pytest.fail(f"{len(g)} rows vs {len(w)} expected; extra {extra}; missing {missing}")
    if summ:
        assert open(summ, "rb").read() == open(os.path.join(d, "expected_summary.txt"), "rb").read()


RANDOM_CASES = [
    dict(seed=201, lens=[120000, 80000], pattern="N" * 21 + "GG", mm=5, per_guide=40),
    dict(seed=202, lens=[100000, 50000, 7], fmt="2bit", pattern="N" * 21 + "RG", dna=2, rna=1, mm=5, per_guide=40,
         n_frac=0.05, gc_drift=0.1),
    dict(seed=203, lens=[90000], pattern="TTTV" + "N" * 23, dna=1, rna=1, mm=4, per_guide=40),
    dict(seed=204, lens=[60000, 40000], pattern="N" * 21 + "NNGRRT", dna=1, rna=1, mm=[3, 6], iupac_frac=0.1,
         sprinkle_chars="RYKMWSBDHVnacgtX*-", with_ids=True),
    dict(seed=205, lens=[70000], pattern="N" * 24 + "NNNNGMTT", dna=1, rna=1, mm=5, per_guide=40),
    dict(seed=206, lens=[50000, 50000], pattern="N" * 20 + "NNAGAAW", dna=1, rna=1, mm=4, per_guide=40),
    dict(seed=207, lens=[30000], pattern="N" * 40 + "NGG", dna=2, rna=2, mm=8, per_guide=40),
    # The CPU-runnable configuration's shape: 4 FASTA records, 10 Mbp, NGG
    # without bulges, 4 guides at mm 4 (and one at 6), planted sites.
    dict(seed=208, lens=[3000000, 2600000, 2400000, 2000000], pattern="N" * 21 + "GG", mm=[4, 4, 4, 6],
         per_guide=60, n_frac=0.01),
    # The longest pattern (62 + DNA bulge 2 = 64 positions: two plane words
    # per window), and windows of exactly one plane word (32, no bulge).
    dict(seed=209, lens=[40000, 30000], pattern="N" * 59 + "NGG", dna=2, rna=1, mm=[8, 12], per_guide=30),
    dict(seed=210, lens=[60000], pattern="N" * 29 + "NRG", mm=6, per_guide=40, iupac_frac=0.05),
    # A 48-position pattern whose guides leave the first 18 spacer bases N:
    # 27 positions that can mismatch, so the bit-sliced comparer takes the
    # two-word windows (68-column class rows).
    dict(seed=211, lens=[80000, 20000], pattern="N" * 45 + "NGG", dna=1, rna=1, mm=5, per_guide=40,
         guides=["N" * 18 + "".join(random.Random(211 + i).choice("ACGT") for _ in range(27)) + "NNN"
                 for i in range(3)]),
    # Thresholds at the edges of the bit-sliced comparer's narrow counters
    # (20-nt guides, 20 slots, 5 count planes: thresholds 4 and 15 fit them,
    # 3 and 16 take the sixth plane).
    dict(seed=212, lens=[20000], pattern="N" * 21 + "RG", dna=1, rna=1, mm=[4, 15], per_guide=20,
         guides=["".join(random.Random(212 + i).choice("ACGT") for _ in range(20)) + "NNN" for i in range(2)]),
    dict(seed=213, lens=[20000], pattern="N" * 21 + "RG", dna=1, rna=1, mm=[3, 16], per_guide=20,
         guides=["".join(random.Random(213 + i).choice("ACGT") for _ in range(20)) + "NNN" for i in range(2)]),
    # More lane programs than one 32-lane chunk (~700 variants, 3 chunks):
    # CTAs of several warps, with narrow counters (21 positions, mm 5) and
    # without (mm 3 among them).
    dict(seed=214, lens=[100000], pattern="N" * 21 + "RG", dna=2, rna=1, mm=5, n_guides=12, per_guide=10),
    dict(seed=215, lens=[100000], pattern="N" * 21 + "RG", dna=2, rna=1, mm=[3, 5], n_guides=12, per_guide=10),
]


@pytest.mark.parametrize("spec", RANDOM_CASES, ids=[str(c["seed"]) for c in RANDOM_CASES])
def test_cli_matches_oracle_random(spec, P, built, oracle, tmp_path):
    inp, _ = cases.make_case(str(tmp_path), **spec)
    a, b = str(tmp_path / "ora.tsv"), str(tmp_path / "gpu.tsv")
    sa, sb = str(tmp_path / "ora_summary.txt"), str(tmp_path / "gpu_summary.txt")
    ra = cases.run_cli(oracle, inp, a, threads=4, summary=sa)
    rb = cases.run_cli(P.CLI_PATH, inp, b, device="G0", summary=sb)
    assert ra.returncode == 0, ra.stderr.decode()
    assert rb.returncode == 0, rb.stderr.decode()
    ta, tb = open(a, "rb").read(), open(b, "rb").read()
    assert len(cases.rows_of(ta)) > 0
    assert ta == tb
    # summary table: counts per (id, bulge type, bulge size, mismatches)
    assert open(sa, "rb").read() == open(sb, "rb").read()


def test_abi_search_matches_golden_and_repeats(P, built, tmp_path):
    """Through the C ABI: same rows twice in a row, and after reloading."""
    case = "nrg_bulge_2bit"
    d = os.path.join(GOLDEN, case)
    inp = golden_input(case, tmp_path)
    want = open(os.path.join(d, "expected.tsv"), "rb").read()
    with P.CasOFFinder(0) as eng:
        eng.read_input_path(inp)
        eng.load_genome_file(eng.chrdir)
        first = eng.search()   # passes captured as a CUDA graph
        second = eng.search()  # graph replayed
        eng.set_profiling(True)
        third = eng.search()   # profiled: passes launched directly
        eng.set_profiling(False)
        assert P.HEADER.encode() + first == want
        assert first == second == third
        nh, nr = eng.last_hit_count()
        assert nr == len(cases.rows_of(want))


def test_abi_text_and_planes_loaders_agree(P, built, tmp_path):
    """load_genome_text / load_genome_planes give the same rows as the file loader."""
    case = "iupac_nngrrt"
    inp = golden_input(case, tmp_path)
    want = open(os.path.join(GOLDEN, case, "expected.tsv"), "rb").read()
    names, seqs = read_fasta(os.path.join(GOLDEN, case, "genome.fa"))
    text, starts = P.reference_text(seqs)
    with P.CasOFFinder(0) as eng:
        eng.read_input_path(inp)
        eng.load_genome_text(text, names, starts)
        assert P.HEADER.encode() + eng.search() == want
        hi, lo, ot, ep, eb = P.pack_text(text)
        eng.load_genome_planes(hi, lo, ot, len(text), ep, eb, names, starts)
        assert P.HEADER.encode() + eng.search() == want


def test_search_planes_streams_like_resident_search(P, built):
    """cof_search_planes (upload of segment s+1 overlapped with the scan of
    segment s) gives the rows of load_genome_planes + cof_search, on a genome
    of several 2^26-position segments, from pageable and from pinned memory;
    afterwards the genome is resident."""
    import random
    rng = random.Random(11)
    lens = [70_000_000, 45_000_000, 33_000_000]
    seqs = [P.synth_record(21, r, n, gc=0.41, n_frac=0.02, n_run_min=100, n_run_max=5000)
            for r, n in enumerate(lens)]
    text, starts = P.reference_text(seqs)
    names = [f"chr{i + 1}" for i in range(len(lens))]
    hi, lo, ot, ep, eb = P.pack_text(text)
    guides = ["".join(rng.choice("ACGT") for _ in range(20)) + "NNN" for _ in range(3)]
    inp = "synthetic\n" + "N" * 21 + "RG 1 1\n" + "".join(f"{g} 5\n" for g in guides)
    with P.CasOFFinder(0) as eng:
        eng.readInputFile(inp)
        eng.load_genome_planes(hi, lo, ot, len(text), ep, eb, names, starts)
        want = eng.search()
        assert len(cases.rows_of(want)) > 100
        # The first search timed the candidate program lengths on a segment;
        # the rows do not depend on the choice.
        sched = eng.schedule()
        assert "tuned:" in sched, sched
        eng.set_autotune(False)
        assert eng.search() == want
        assert "tuned:" not in eng.schedule()
        eng.set_autotune(True)
        got = P._bytes_at(*eng.search_planes_view(hi, lo, ot, len(text), ep, eb, names, starts))
        assert got == want
        torch = pytest.importorskip("torch")
        W = P.plane_words(len(text))
        pinned = torch.empty(3 * W, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        pinned[:W], pinned[W:2 * W], pinned[2 * W:] = hi, lo, ot
        got = P._bytes_at(*eng.search_planes_view(pinned[:W], pinned[W:2 * W], pinned[2 * W:], len(text), ep, eb,
                                                  names, starts))
        assert got == want
        pinned[:] = 0  # the genome is resident: the host planes are no longer read
        assert eng.search() == want


def test_hit_buffer_growth_with_captured_passes(P, built):
    """More hits than the first hit buffer holds: the passes are captured
    again for the larger buffer, and the rows equal the directly launched
    (profiled) search's."""
    seqs = [P.synth_record(5, 0, 15_000_000, gc=0.41)]
    text, starts = P.reference_text(seqs)
    hi, lo, ot, ep, eb = P.pack_text(text)
    inp = "synthetic\n" + "N" * 20 + "NGG\n" + "ACGTACGTACGTACGTACGT" + "NNN 20\n"
    with P.CasOFFinder(0) as eng:
        eng.readInputFile(inp)
        eng.load_genome_planes(hi, lo, ot, len(text), ep, eb, ["chr1"], starts)
        a = eng.search()
        nh, nr = eng.last_hit_count()
        assert nh > (1 << 20)
        eng.set_profiling(True)
        b = eng.search()
        eng.set_profiling(False)
        assert a == b
        assert eng.search() == a
        # The same rows streamed in chunks of 2^20 hits (two chunks here).
        parts = []
        assert eng.search_stream(parts.append) == len(a)
        assert len(parts) == 2 and b"".join(parts) == a

        def refuse(chunk):
            raise IOError("disk full")
        with pytest.raises(P.CofError) as e:
            eng.search_stream(refuse)
        assert e.value.status == 5  # COF_ERR_IO
        assert eng.search() == a    # the handle stays usable


def read_fasta(path):
    names, seqs = [], []
    for line in open(path, "rb").read().split(b"\n"):
        line = line.rstrip(b"\r")
        if line.startswith(b">"):
            names.append(line[1:])
            seqs.append(bytearray())
        elif line:
            seqs[-1] += line
    return names, seqs


def test_kernel_level_chunk_abi(P, built, tmp_path):
    """cof_finder_chunk / cof_comparer_chunk (the OpenCL kernels' contracts)
    against the numpy restatement of finder_cpu/comparer_cpu (cases.py,
    itself checked against the reference's rows) on a small chunk: concrete,
    IUPAC-coded and 2-word compare strings."""
    names, seqs = read_fasta(os.path.join(GOLDEN, "ngg_fasta", "genome.fa"))
    text, _ = P.reference_text(seqs)
    text = text[:30000]
    rc_tab = bytes.maketrans(b"ACGTRYKMHDBV", b"TGCAYRMKDHVB")
    with P.CasOFFinder(0) as eng:
        for pattern, queries in (
                (b"N" * 21 + b"GG", [(b"GGCCGACCTGTCGCTGACGCNNN", 9), (b"GGCCRACCTGYCGCTGASGCNNN", 8),
                                     (b"ACGTHBVDACGTWSKMACGTNNN", 12)]),
                (b"N" * 45 + b"NGG", [(b"GGCCGACCTGTCGCTGACGCAGTCRYACGGTTACGATCGATCGAANNN", 26)])):
            L = len(pattern)
            worksize = len(text) - L + 1
            loci, flag = eng.finder_chunk(text, worksize, pattern + pattern[::-1].translate(rc_tab), L)
            exp_loci, exp_flag = cases.restate_finder(text, pattern)
            assert loci.tolist() == exp_loci.tolist()
            assert flag.tolist() == exp_flag.tolist()
            for comp, thr in queries:
                mm_loci, mm_count, direction = eng.comparer_chunk(text, loci, flag, comp, thr)
                got = list(zip(mm_loci.tolist(), [d == ord("-") for d in direction], mm_count.tolist()))
                assert got == cases.restate_comparer(text, loci, flag, comp, thr), comp
                assert len(got) > 0, comp


@pytest.mark.parametrize("spec", RANDOM_CASES[:5], ids=[str(c["seed"]) for c in RANDOM_CASES[:5]])
def test_both_comparers_identical(spec, P, built, oracle, tmp_path):
    """The popcount and the bit-sliced comparer give the same rows as the oracle."""
    inp, _ = cases.make_case(str(tmp_path), **spec)
    a = str(tmp_path / "ora.tsv")
    assert cases.run_cli(oracle, inp, a, threads=4).returncode == 0
    want = open(a, "rb").read()
    with P.CasOFFinder(0) as eng:
        eng.read_input_path(inp)
        eng.load_genome_file(eng.chrdir)
        for kind in (1, 2, 0):
            eng.set_comparer(kind)
            assert P.HEADER.encode() + eng.search() == want, f"comparer {kind}"


def test_positions_past_2_to_the_32(P, built, oracle, tmp_path):
    """A genome longer than 2^32 bytes: a first record of N up to just below
    2^32, then a 1 Mbp record with planted sites on both sides of position
    2^32.  Rows carry record-relative locations, so the GPU rows must equal
    the oracle's rows for the second record searched alone."""
    import random
    rng = random.Random(232)
    pattern, dna, rna = "N" * 21 + "RG", 1, 1
    guides = [("".join(rng.choice("ACGT") for _ in range(20)) + "NNN", 5) for _ in range(3)]
    rec = P.synth_record(232, 0, 1_000_000, n_frac=0.01, n_run_min=50, n_run_max=500)
    cases.plant_sites(rng, [rec], pattern, [g for g, _ in guides], 60, 5, dna, rna)
    start = (1 << 32) - (1 << 19)  # word-aligned start of the second record
    n = start + len(rec)
    W = P.plane_words(n)
    hi, lo, ot = (np.zeros(W, np.uint32) for _ in range(3))
    ot[:start // 32] = 0xFFFFFFFF  # the N record ...
    sep = start - 1
    lo[sep // 32] |= np.uint32(1 << (sep % 32))  # ... and the ';' before chrX
    rh, rl, ro, rexc, _ = P.pack_text(bytes(rec))
    assert rexc.size == 0
    k = (len(rec) + 31) // 32
    hi[start // 32:start // 32 + k], lo[start // 32:start // 32 + k], ot[start // 32:start // 32 + k] = \
        rh[:k], rl[:k], ro[:k]
    fa = str(tmp_path / "rec.fa")
    P.write_fasta(fa, ["chrX"], [bytes(rec)])
    text = f"{fa}\n{pattern} {dna} {rna}\n" + "".join(f"{g} {mm}\n" for g, mm in guides)
    inp = str(tmp_path / "in.txt")
    open(inp, "w").write(text)
    out = str(tmp_path / "ora.tsv")
    r = cases.run_cli(oracle, inp, out, threads=4)
    assert r.returncode == 0, r.stderr.decode()
    want = open(out, "rb").read()
    rows = cases.rows_of(want)
    assert len(rows) > 50
    locs = [int(x.split(b"\t")[5]) for x in rows]
    assert min(locs) < (1 << 19) < max(locs)  # hits on both sides of 2^32
    # The plane words past the end hold zeros (bases T): the scan must stop
    # at the genome's end by itself.
    assert not ot[n // 32 + 1:].any()
    with P.CasOFFinder(0) as eng:
        eng.readInputFile(text)
        eng.load_genome_planes(hi, lo, ot, n, None, None, ["big", "chrX"], [0, start])
        assert eng.genome_info() == (n, 2)
        got = eng.search()
        assert P.HEADER.encode() + got == want
        # Planes without the separator before a record are refused.
        lo[sep // 32] &= np.uint32(~(1 << (sep % 32)) & 0xFFFFFFFF)
        with pytest.raises(P.CofError) as e:
            eng.load_genome_planes(hi, lo, ot, n, None, None, ["big", "chrX"], [0, start])
        assert e.value.status == 2 and "separator" in e.value.message


def test_cli_directory_matches_oracle(P, built, oracle, tmp_path):
    """Line 1 naming a directory: every genome file in readdir order (a FASTA
    file, a 2BIT file, a file that is neither), rows written file by file,
    the summary counted over all files -- as the reference's main.cpp walks
    it.  Each file replaces the resident genome, so each search recaptures
    its passes and streams its rows again."""
    import random
    rng = random.Random(77)
    pattern, dna, rna = "N" * 21 + "RG", 1, 1
    guides = ["".join(rng.choice("ACGT") for _ in range(20)) + "NNN" for _ in range(3)]
    recs = [P.synth_record(177, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
            for r, n in enumerate([300000, 80000, 200000, 5000])]
    cases.plant_sites(rng, recs, pattern, guides, 40, 5, dna, rna)
    d = tmp_path / "genome"
    d.mkdir()
    P.write_fasta(str(d / "a.fa"), ["chr1", "chr2"], [bytes(r) for r in recs[:2]])
    cases.write_genome(str(d / "b.2bit"), "2bit", ["chr3", "chr4"], recs[2:])
    (d / "readme.txt").write_text("not a genome\n")
    (d / "c.fa").write_text(">empty\n")
    inp = str(tmp_path / "in.txt")
    open(inp, "w").write(f"{d}\n{pattern} {dna} {rna}\n" + "".join(f"{g} 5\n" for g in guides))
    a, b = str(tmp_path / "ora.tsv"), str(tmp_path / "gpu.tsv")
    sa, sb = str(tmp_path / "ora_summary.txt"), str(tmp_path / "gpu_summary.txt")
    ra = cases.run_cli(oracle, inp, a, threads=4, summary=sa)
    rb = cases.run_cli(P.CLI_PATH, inp, b, device="G0", summary=sb)
    assert ra.returncode == 0, ra.stderr.decode()
    assert rb.returncode == 0, rb.stderr.decode()
    ta = open(a, "rb").read()
    chroms = {r.split(b"\t")[4] for r in cases.rows_of(ta)}
    assert {b"chr1", b"chr3"} <= chroms  # rows from both genome files
    assert ta == open(b, "rb").read()
    assert open(sa, "rb").read() == open(sb, "rb").read()


def test_cli_gzip_output(P, built, tmp_path):
    """An output name ending in .gz: the same bytes, gzip-compressed."""
    import gzip
    case = "nrg_bulge_2bit"
    d = os.path.join(GOLDEN, case)
    inp = golden_input(case, tmp_path)
    out = str(tmp_path / "gpu.tsv.gz")
    r = cases.run_cli(P.CLI_PATH, inp, out, device="G0")
    assert r.returncode == 0, r.stderr.decode()
    assert gzip.decompress(open(out, "rb").read()) == open(os.path.join(d, "expected.tsv"), "rb").read()
