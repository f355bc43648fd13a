"""Served mode: requests admitted while others run (continuous batching over
the genome ring) give exactly the rows of each input file searched alone."""
import random
import threading

import pytest

import cases
from test_gpu_batch import batch_inputs

pytestmark = pytest.mark.gpu


def make_genome_and_requests(P, tmp_path):
    rng = random.Random(55)
    seqs = [P.synth_record(512, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
            for r, n in enumerate([200000, 120000])]
    genome = str(tmp_path / "genome.fa")
    texts = batch_inputs(rng, genome)
    for t in texts:
        lines = t.strip().split("\n")
        pat = lines[1].split()
        dna = int(pat[1]) if len(pat) == 3 else 0
        rna = int(pat[2]) if len(pat) == 3 else 0
        cases.plant_sites(rng, seqs, pat[0], [l.split()[0] for l in lines[2:]], 20, 6, dna, rna)
    P.write_fasta(genome, ["chr1", "chr2"], seqs)
    return genome, texts


def oracle_rows(oracle, tmp_path, texts):
    want = []
    for j, t in enumerate(texts):
        path = str(tmp_path / f"req{j}.txt")
        open(path, "w").write(t)
        out = str(tmp_path / f"req{j}.tsv")
        r = cases.run_cli(oracle, path, out, threads=4)
        assert r.returncode == 0, r.stderr.decode()
        want.append(open(out, "rb").read())
    return want


def test_server_mix_equals_alone(P, built, oracle, tmp_path):
    genome, texts = make_genome_and_requests(P, tmp_path)
    want = oracle_rows(oracle, tmp_path, texts)
    assert all(len(cases.rows_of(w)) > 0 for w in want)
    with P.CasOFFinder(0) as eng:
        # 32 Ki positions per segment: a ring of 10 segments over this genome,
        # and a small variant budget, so requests join the ring mid-way while
        # others are running.
        eng.load_genome_file(genome)
        with P.Server(eng, max_active_variants=250, segment_positions=1 << 15) as srv:
            tickets = [None] * len(texts)

            def client():  # back to back: later requests arrive while the first ones run
                for j, t in enumerate(texts):
                    tickets[j] = srv.submit(t)

            th = threading.Thread(target=client)
            th.start()
            th.join()
            got = [srv.wait(t) for t in tickets]
            stats = srv.stats()
        for j in range(len(texts)):
            rows, lat = got[j]
            assert lat >= 0
            assert P.HEADER.encode() + rows == want[j], f"request {j} in the mix"
        assert stats["admitted"] == len(texts) and stats["completed"] == len(texts)
        assert stats["max_active"] >= 2  # requests ran together
        assert stats["steps"] > 10  # more steps than one ring: requests joined mid-ring
        # Each request alone on a fresh server: the same rows.
        with P.Server(eng, segment_positions=1 << 15) as srv:
            for j in (0, 3):
                rows, _ = srv.wait(srv.submit(texts[j]))
                assert P.HEADER.encode() + rows == want[j], f"request {j} alone"


def test_server_step_segments_keep_rows(P, built, oracle, tmp_path):
    """Steps of 1, 3 and 7 ring segments (a ring of 10): requests that join
    between steps still see each segment exactly once, so the rows are those
    of each input file alone."""
    genome, texts = make_genome_and_requests(P, tmp_path)
    texts = texts[:4]
    want = oracle_rows(oracle, tmp_path, texts)
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        for k in (1, 3, 7):
            with P.Server(eng, max_active_variants=250, segment_positions=1 << 15) as srv:
                srv.set_step_segments(k)
                tickets = [srv.submit(t) for t in texts]
                got = [srv.wait(t) for t in tickets]
                stats = srv.stats()
            for j, (rows, _) in enumerate(got):
                assert P.HEADER.encode() + rows == want[j], f"request {j}, {k} segments per step"
            assert stats["completed"] == len(texts)


def test_server_burst_is_formatted_together(P, built, oracle, tmp_path):
    """Requests submitted back to back share the ring; those that complete at
    the same step are formatted as one batch (one sort and one row pass over
    all of their hits, each request's byte range copied out on its own); each
    still gets exactly its own rows."""
    genome, texts = make_genome_and_requests(P, tmp_path)
    want = oracle_rows(oracle, tmp_path, texts)
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        with P.Server(eng, segment_positions=1 << 15) as srv:
            tickets = [srv.submit(t) for t in texts]
            got = [srv.wait(t) for t in tickets]
            stats = srv.stats()
        for j, (rows, _) in enumerate(got):
            assert P.HEADER.encode() + rows == want[j], f"request {j} of the burst"
        assert stats["completed"] == len(texts)
        assert stats["max_active"] >= 2  # requests shared the ring


def test_server_admits_by_hit_memory(P, built, oracle, tmp_path):
    """Admission by device memory: each running request is charged at least
    its hit reservation against hit_buffer_bytes, so a reservation of half the
    budget lets at most two requests run together, and one of the whole budget
    only one; the rows stay those of each input file alone."""
    genome, texts = make_genome_and_requests(P, tmp_path)
    texts = texts[:6]
    want = oracle_rows(oracle, tmp_path, texts)
    budget = 1 << 20
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        for reserve, most in ((budget // 2, 2), (budget, 1)):
            with P.Server(eng, hit_buffer_bytes=budget, segment_positions=1 << 15) as srv:
                srv.set_hit_reserve(reserve)
                tickets = [srv.submit(t) for t in texts]
                got = [srv.wait(t) for t in tickets]
                stats, mem = srv.stats(), srv.memory()
            for j, (rows, _) in enumerate(got):
                assert P.HEADER.encode() + rows == want[j], f"request {j}, reservation {reserve}"
            assert stats["completed"] == len(texts)
            assert 1 <= stats["max_active"] <= most, stats
            assert mem["queue_bytes"] == 2 * 2 * (1 << 15) * 4  # two queues, two entries per position
            assert 0 < mem["max_held_hit_bytes"] <= budget


def test_server_rejects_bad_input_and_times_out_cleanly(P, built, tmp_path):
    genome, texts = make_genome_and_requests(P, tmp_path)
    with P.CasOFFinder(0) as eng:
        eng.load_genome_file(genome)
        with P.Server(eng) as srv:
            with pytest.raises(P.CofError) as e:
                srv.submit(f"{genome}\nNNNNNNNNNNNNNNNNNNNNNGG\nACGT 3 x y\n")
            assert "Malformed" in e.value.message
            t = srv.submit(texts[0])
            r = srv.wait(t, timeout_ms=0)  # may or may not be done already
            if r is None:
                r = srv.wait(t)
            assert r is not None


def test_router_keeps_genome_sets_resident(P, built, oracle, tmp_path):
    """Requests for two genomes -- a directory of a FASTA file, a 2BIT file and
    a file that is neither, and a single FASTA file -- sent through one router
    from two threads: each request's rows are the oracle's for its input file
    (the directory's files in readdir order, the non-genome file skipped)."""
    rng = random.Random(66)
    seqs_a = [P.synth_record(613, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
              for r, n in enumerate([120000, 60000, 90000])]
    seqs_b = [P.synth_record(614, r, n, n_frac=0.01, n_run_min=50, n_run_max=500)
              for r, n in enumerate([150000, 40000])]
    dir_a = tmp_path / "genome_a"
    dir_a.mkdir()
    file_b = str(tmp_path / "genome_b.fa")
    texts = []
    for genome, seqs in ((str(dir_a), seqs_a), (file_b, seqs_b)):
        for t in batch_inputs(rng, genome):
            lines = t.strip().split("\n")
            pat = lines[1].split()
            dna = int(pat[1]) if len(pat) == 3 else 0
            rna = int(pat[2]) if len(pat) == 3 else 0
            cases.plant_sites(rng, seqs, pat[0], [l.split()[0] for l in lines[2:]], 15, 6, dna, rna)
            texts.append(t)
    P.write_fasta(str(dir_a / "part1.fa"), ["chr1", "chr2"], seqs_a[:2])
    cases.write_genome(str(dir_a / "part2.2bit"), "2bit", ["chr3"], seqs_a[2:])
    (dir_a / "notes.txt").write_text("not a genome\n")
    P.write_fasta(file_b, ["chrB1", "chrB2"], seqs_b)
    want = oracle_rows(oracle, tmp_path, texts)
    assert all(len(cases.rows_of(w)) > 0 for w in want)
    order = list(range(len(texts)))
    rng.shuffle(order)
    with P.Router(0, max_active_variants=300, segment_positions=1 << 15, auto_load=True) as router:
        assert router.add_genome(str(dir_a)) == 2  # notes.txt skipped
        tickets = {}

        def client(js):
            for j in js:
                tickets[j] = router.submit(texts[j])  # genome_b loads on its first request

        ths = [threading.Thread(target=client, args=(order[k::2],)) for k in range(2)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        got = {j: router.wait(t) for j, t in tickets.items()}
        assert router.genomes() == (2, 3)
        for j in range(len(texts)):
            rows, lat = got[j]
            assert lat >= 0
            assert P.HEADER.encode() + rows == want[j], f"request {j}"
        # A genome with no requests outstanding can be dropped, and comes back
        # on the next request that names it.
        router.drop_genome(file_b)
        assert router.genomes() == (1, 2)
        j = len(texts) - 1
        rows, _ = router.wait(router.submit(texts[j]))
        assert P.HEADER.encode() + rows == want[j]
    with P.Router(0) as router:  # without auto_load an unknown genome is refused
        with pytest.raises(P.CofError) as e:
            router.submit(texts[0])
        assert e.value.status == 6 and "not resident" in e.value.message
