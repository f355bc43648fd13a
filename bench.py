#!/usr/bin/env python3
"""Benchmark: guide-Gbp/s of the plain Cas-OFFinder search on one GB300.

Workload (the full-scale plain configuration): a synthetic 3.1 Gbp genome of 24
records (lengths log-uniform in 47-249 Mbp, rescaled to 3.1 Gbp), 41% GC with
a +-10% GC drift per 100 kbp window and 5% N in runs of 1-100 kbp; pattern
NNNNNNNNNNNNNNNNNNNNNRG with DNA bulge 2 and RNA bulge 1; 4 random 20-nt
guides + NNN with at most 5 mismatches.  All inputs are seeded.

One step = one full search of the genome (PAM scan, compare, sort, row
formatting on the GPU, rows copied to host memory).
  value : steps with the packed genome already resident in HBM.
  e2e   : steps through the C ABI from host buffers: each step uploads the
          genome planes from pinned host memory and searches them in one call
          (cof_search_planes: the upload runs ahead on a copy stream while
          the segments already copied are scanned), and copies the rows back.
The genome planes (1.16 GB) are larger than L2, so no flush is needed between
steps.  Timing: CUDA events on the engine's stream (cof_timer_start/stop),
after warm-up steps, max over ranks.  Under torchrun each rank runs an
independent replica on its own GPU (weak scaling; the search has no
cross-GPU exchange).

--impl reference times the reference's own CPU path on the host cores instead
(its finder_cpu/comparer_cpu through its unmodified host code, device C, built
from its sources by oracle/build_ref.py; the oracle's C++ restatement only
where that build is absent), on the first 20 Mbp of the same genome, rate
per base extrapolated to the whole genome.  That arm loads no library of this
package: its genome file comes from the standalone cof-synth writer.

verify (on by default, --no-verify skips it): after the timed legs the oracle
(the CPU restatement, every host core) searches the same inputs, and the GPU
rows are compared byte for byte: the whole 3.1 Gbp genome for the plain
search, and samples of the timed batched, PAM-variety and served searches
over the genome's leading records.
"""
import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PATTERN = "N" * 21 + "RG"
DNA, RNA, MM, N_GUIDES = 2, 1, 5, 4
GENOME_SEED = 2
GUIDE_SEED = 3
METRIC = "guide-Gbp/s (bit-exact hits) plain vs batched-served; p50/p99 request latency"
WORKLOAD = ("plain: 3.1 Gbp synthetic genome (24 records, 41% GC +-10% drift, 5% N), "
            "NNNNNNNNNNNNNNNNNNNNNRG dna 2 rna 1, 4 random 20-nt guides + NNN, mm 5")


def pkg():
    from pkgload import pkg as _p
    return _p()


def make_guides(seed=GUIDE_SEED, n=N_GUIDES):
    import random
    rng = random.Random(seed)
    return ["".join(rng.choice("ACGT") for _ in range(20)) + "NNN" for _ in range(n)]


def batched_jobs(seed=5, n=1024, genome_path="synthetic"):
    """The 1,024-guide mixed workload: one input file per guide, spacer 20-24
    random bases with 2% IUPAC degenerate codes, PAM NGG or NRG (50/50), max
    mismatches 3-6, DNA bulge 0-2, RNA bulge 0-1 (all uniform)."""
    import random
    rng = random.Random(seed)
    texts = []
    for _ in range(n):
        spacer = rng.randint(20, 24)
        pam = rng.choice(["NGG", "NRG"])
        mm, dna, rna = rng.randint(3, 6), rng.randint(0, 2), rng.randint(0, 1)
        guide = "".join(rng.choice("ACGT") if rng.random() >= 0.02 else rng.choice("RYKMWSBDHV")
                        for _ in range(spacer)) + "NNN"
        pattern = "N" * spacer + pam
        line2 = pattern + (f" {dna} {rna}" if (dna or rna) else "")
        texts.append(f"{genome_path}\n{line2}\n{guide} {mm}\n")
    return texts


PAM_SETS = [("NNGRRT", 21, False), ("NNNNGMTT", 24, False), ("NNAGAAW", 20, False), ("TTTV", 23, True)]


def pam_variety_jobs(seed=7, per_set=256, genome_path="synthetic"):
    """PAM and orientation variety: four input files of 256 random guides each
    (NNGRRT with 21-nt spacers, NNNNGMTT with 24, NNAGAAW with 20, and the 5'
    PAM TTTV with 23), max mismatches 4, DNA bulge 1, RNA bulge 1."""
    import random
    rng = random.Random(seed)
    texts = []
    for pam, spacer, pam5 in PAM_SETS:
        pattern = (pam + "N" * spacer) if pam5 else ("N" * spacer + pam)
        lines = [genome_path, pattern + " 1 1"]
        for _ in range(per_set):
            g = "".join(rng.choice("ACGT") for _ in range(spacer))
            lines.append((("N" * len(pam) + g) if pam5 else (g + "N" * len(pam))) + " 4")
        texts.append("\n".join(lines) + "\n")
    return texts


SERVED_PAMS = [("NGG", 20, False), ("NRG", 20, False), ("NNGRRT", 21, False), ("TTTV", 23, True)]


def served_requests(seed=9, n=12, genome_path="synthetic"):
    """Requests of the served workload: 1-512 guides (log-uniform), a PAM from
    {NGG, NRG, NNGRRT, TTTV}, max mismatches 2-6, DNA and RNA bulges 0-2."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        pam, spacer, pam5 = rng.choice(SERVED_PAMS)
        ng = int(round(math.exp(rng.uniform(0.0, math.log(512)))))
        dna, rna = rng.randint(0, 2), rng.randint(0, 2)
        pattern = (pam + "N" * spacer) if pam5 else ("N" * spacer + pam)
        lines = [genome_path, pattern + (f" {dna} {rna}" if (dna or rna) else "")]
        for _ in range(ng):
            sp = "".join(rng.choice("ACGT") for _ in range(spacer))
            g = ("N" * len(pam) + sp) if pam5 else (sp + "N" * len(pam))
            lines.append(f"{g} {rng.randint(2, 6)}")
        out.append(("\n".join(lines) + "\n", ng))
    return out


def percentile(xs, q):
    """Nearest-rank percentile (q in [0, 1]) of a list of numbers."""
    ys = sorted(xs)
    return ys[min(len(ys) - 1, max(0, int(round(q * (len(ys) - 1)))))]


def run_served(P, eng, lens, args, capture=None):
    """Served mode: the same request list arriving as a Poisson stream at each
    rate; per rate p50/p99 latency (submit to rows in host memory) over every
    request, where each request's latency went (admission, table build, ring
    pass, formatting), and whole-run guide-Gbp/s, against the plain path run
    once per request."""
    import ctypes
    import random
    import statistics
    import threading
    gbp = sum(lens) / 1e9
    reqs = served_requests(n=args.served_requests)
    guides = sum(ng for _, ng in reqs)
    # Plain: each request alone through cof_read_input + cof_search.
    eng.readInputFile(reqs[0][0])
    eng.search_view()
    plain_ms = []
    for text, _ in reqs:
        eng.readInputFile(text)
        eng.synchronize()
        eng.timer_start()
        eng.search_view()
        plain_ms.append(eng.timer_stop())
    out = {"workload": f"{len(reqs)} requests per rate, 1-512 guides each (log-uniform; {guides} guides), PAM NGG/"
                       "NRG/NNGRRT/TTTV, mm 2-6, DNA/RNA bulge 0-2, on the same 3.1 Gbp genome",
           "plain_value": guides * gbp / (sum(plain_ms) / 1e3), "unit": "guide-Gbp/s",
           "plain_latency_ms": {"p50": statistics.median(plain_ms), "p99": percentile(plain_ms, 0.99),
                                "max": max(plain_ms)}, "rates": []}
    keep = [f"chr{i + 1}" for i in range(VERIFY_SERVED_RECORDS)]
    pick = sorted(range(len(reqs)), key=lambda j: (reqs[j][1], j))[:VERIFY_SERVED_REQUESTS]
    stages = ("admission", "build", "ring", "format")
    for rate in args.served_rates:
        rng = random.Random(int(rate * 1000))
        lat, parts = [None] * len(reqs), [None] * len(reqs)
        kept = {}
        verify_here = capture is not None and rate == args.served_rates[-1]
        with P.Server(eng) as srv:
            t0 = time.perf_counter()

            # Each arrival is submitted from its own thread, as a concurrent
            # caller would (submit parses the input file on the caller's
            # thread), which then waits for its rows and releases them.
            def client(j, at):
                d = at - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                t = srv.submit(reqs[j][0])
                addr, n, lat[j] = srv.wait_view(t)
                parts[j] = srv.timing(t)
                if verify_here and j in pick:
                    kept[j] = rows_of_records(ctypes.string_at(addr, n), keep)
                srv.release(t)

            threads, at = [], t0
            for j in range(len(reqs)):
                at += rng.expovariate(rate)
                threads.append(threading.Thread(target=client, args=(j, at)))
                threads[-1].start()
            for th in threads:
                th.join()
            span = time.perf_counter() - t0
            st = srv.stats()
        if verify_here:
            capture["served"] = {"records": VERIFY_SERVED_RECORDS, "rate": rate, "rows": kept}
            capture["served_n"] = len(reqs)
        out["rates"].append({
            "arrivals_per_s": rate, "requests": len(reqs), "p50_ms": statistics.median(lat),
            "p99_ms": percentile(lat, 0.99), "value": guides * gbp / span, "makespan_s": span,
            "max_active": st["max_active"], "ring_steps": st["steps"],
            "latency_parts_ms": {k: {"p50": statistics.median(p[k] for p in parts),
                                     "mean": statistics.fmean(p[k] for p in parts)} for k in stages}})
    out["value"] = max(r["value"] for r in out["rates"])
    out["speedup_vs_plain"] = out["value"] / out["plain_value"]
    out["burst_1024"] = run_served_burst(P, eng, lens)
    return out


def run_served_burst(P, eng, lens):
    """The 1,024-guide mixed workload (one single-guide input file per guide)
    submitted to the server at once as 1,024 requests: whole-run guide-Gbp/s
    and latency, against the same input files searched one after another on
    the plain path (a sample of 32 timed)."""
    import statistics
    import threading
    gbp = sum(lens) / 1e9
    texts = batched_jobs()
    eng.readInputFile(texts[0])
    eng.search_view()
    eng.synchronize()
    eng.timer_start()
    for t in texts[:32]:
        eng.readInputFile(t)
        eng.search_view()
    plain_ms = eng.timer_stop() / 32
    lat, parts = [None] * len(texts), [None] * len(texts)
    with P.Server(eng) as srv:
        t0 = time.perf_counter()
        tickets = [srv.submit(t) for t in texts]

        def waiter(lo, hi):
            for j in range(lo, hi):
                lat[j] = srv.wait_view(tickets[j])[2]
                parts[j] = srv.timing(tickets[j])
                srv.release(tickets[j])

        ths = [threading.Thread(target=waiter, args=(i * 128, (i + 1) * 128)) for i in range(len(texts) // 128)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        span = time.perf_counter() - t0
        st = srv.stats()
    value = len(texts) * gbp / span
    plain_value = gbp / (plain_ms / 1e3)
    return {"workload": "the 1,024 single-guide input files of the batched leg, submitted at once as requests",
            "value": value, "unit": "guide-Gbp/s", "makespan_s": span, "p50_ms": statistics.median(lat),
            "p99_ms": percentile(lat, 0.99), "max_active": st["max_active"], "ring_steps": st["steps"],
            "latency_parts_ms": {k: {"p50": statistics.median(p[k] for p in parts),
                                     "mean": statistics.fmean(p[k] for p in parts)}
                                 for k in ("admission", "build", "ring", "format")},
            "plain_value": plain_value,
            "speedup_vs_plain": value / plain_value}


def input_text(genome_path, guides):
    return f"{genome_path}\n{PATTERN} {DNA} {RNA}\n" + "".join(f"{g} {MM}\n" for g in guides)


# The synthetic genome: 41% GC with a +-10% drift per 100 kbp window, 5% N in
# runs of 1-100 kbp (cofx_synth_record / cof-synth arguments).
GENOME_ARGS = (0.41, 0.10, 100000, 0.05, 1000, 100000)


def genome_lengths(total_bp, n_records=24, seed=GENOME_SEED, lo=47_000_000, hi=249_000_000):
    """Record lengths drawn log-uniform in [lo, hi], rescaled to sum to
    total_bp (numpy only; the same draw as the package's record_lengths)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(np.log(lo), np.log(hi), n_records))
    lens = np.floor(raw / raw.sum() * int(total_bp)).astype(np.int64)
    lens[-1] += int(total_bp) - lens.sum()
    return [int(x) for x in lens]


def synth_binary():
    """The standalone genome writer (compiled on demand; no CUDA)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_cof_build", os.path.join(ROOT, "cas-offinder_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_synth()


def write_genome(path, lens, records=None, limit=None, seed=GENOME_SEED):
    """Writes the synthetic genome (records chr1.. of lengths `lens`; only the
    first `records` of them, or only its first `limit` positions) as FASTA, or
    as 2BIT when path ends in .2bit, with cof-synth; returns path."""
    keep = lens[:records] if records else lens
    cmd = [synth_binary()] + (["--limit", str(int(limit))] if limit else []) + \
        [path, str(seed)] + [str(x) for x in GENOME_ARGS] + [f"chr{i + 1}:{n}" for i, n in enumerate(keep)]
    subprocess.run(cmd, check=True)
    return path


def build_genome(P, total_bp, n_records=24, seed=GENOME_SEED, prefix_bp=None):
    """The synthetic genome as the reference's string (records joined by ';').
    prefix_bp: only the leading records that cover that many positions, each
    at its full length (a record's N runs depend on its length), so the
    prefix is byte for byte that of the whole genome."""
    import ctypes
    lens = P.record_lengths(seed, n_records, int(total_bp))
    if prefix_bp is not None:
        keep, covered = 0, 0
        while keep < len(lens) and covered < prefix_bp:
            covered += lens[keep] + 1
            keep += 1
        lens, n_records = lens[:max(keep, 1)], max(keep, 1)
    n = sum(lens) + n_records - 1
    buf = bytearray(n)
    base = ctypes.addressof((ctypes.c_char * n).from_buffer(buf))
    starts, pos = [], 0
    for r, ln in enumerate(lens):
        if r:
            buf[pos] = ord(";")
            pos += 1
        starts.append(pos)
        P.lib().cofx_synth_record(seed, r, ln, *GENOME_ARGS, base + pos)
        pos += ln
    names = [f"chr{r + 1}" for r in range(n_records)]
    return buf, names, starts, lens


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.index = index

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # Timing starts once sampling runs, so nvidia-smi's start-up
            # stays outside the timed region.
            t0 = time.time()
            while time.time() - t0 < 5.0 and self.proc.poll() is None:
                if os.path.exists(self.path) and os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        try:
            rows = [l.split(", ") for l in open(self.path).read().strip().splitlines() if l.strip()]
        except OSError:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_binaries():
    """{'reference': path or None, 'port': path or None}: the reference built
    from its own sources on this machine (oracle/build_ref.py; absent where
    no staged copy of its sources exists) and the oracle's C++ restatement.
    Neither loads a library of this package."""
    import build_oracle
    port, ref = build_oracle.build(with_reference=True)
    out = {"reference": None, "port": None}
    for kind, cand in (("reference", ref), ("port", port)):
        if cand and os.path.exists(cand):
            try:
                if subprocess.run([cand], capture_output=True, timeout=30).returncode == 0:
                    out[kind] = cand
            except (OSError, subprocess.TimeoutExpired):
                continue
    if not out["port"] and not out["reference"]:
        raise RuntimeError("no CPU implementation available")
    return out


def cpu_run(binary, text, threads, workdir, tag="cpu"):
    """Runs a CPU implementation (reference argv: input C output) on one input
    file; returns (seconds, output bytes)."""
    inp = os.path.join(workdir, f"{tag}_input.txt")
    out = os.path.join(workdir, f"{tag}_out.tsv")
    with open(inp, "w") as f:
        f.write(text)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    t0 = time.perf_counter()
    r = subprocess.run([binary, inp, "C", out], env=env, capture_output=True)
    dt = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(f"{binary} failed: " + r.stderr.decode()[-2000:])
    with open(out, "rb") as f:
        data = f.read()
    os.remove(out)
    return dt, data


def count_rows(data):
    return sum(1 for l in data.split(b"\n") if l and not l.startswith(b"#"))


def cpu_plain_sample(binary, lens, sample_bp, guides, threads, workdir):
    """The plain workload on the first `sample_bp` positions of the genome:
    (seconds, rows, guide-Gbp/s extrapolated per base to the whole genome)."""
    fa = os.path.join(workdir, f"sample_{sample_bp}.fa")
    if not os.path.exists(fa):
        write_genome(fa, lens, limit=sample_bp)
    dt, out = cpu_run(binary, input_text(fa, guides), threads, workdir, "plain")
    return dt, count_rows(out), len(guides) * (sample_bp / 1e9) / dt


def run_reference_arm(args, world, rank):
    """The reference's own CPU path on this machine's cores, on the plain
    workload's first 20 Mbp (rank 0 only).  Loads no library of this package."""
    if rank != 0:
        return
    tools = cpu_binaries()
    kind = "reference" if tools["reference"] else "port"
    binary = tools[kind]
    guides = make_guides()
    lens = genome_lengths(args.genome_gbp * 1e9)
    sample_bp = min(int(args.sample_mbp * 1e6), sum(lens) + len(lens) - 1)
    threads = os.cpu_count() or 1
    times = []
    with tempfile.TemporaryDirectory() as tmp:
        for i in range(args.warmup + args.steps):
            dt, rows, _ = cpu_plain_sample(binary, lens, sample_bp, guides, threads, tmp)
            if i >= args.warmup:
                times.append(dt)
    total = sum(times)
    gbp = sample_bp / 1e9
    value = N_GUIDES * gbp * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "guide-Gbp/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_bp": sample_bp},
        "cpu_baseline": {"value": value, "unit": "guide-Gbp/s", "cores": threads, "kind": kind,
                         "program": os.path.relpath(binary, ROOT),
                         "sample": f"first {sample_bp} bp of the same genome and input ({rows} rows per step); "
                                   f"guide-Gbp/s extrapolated per base to the whole genome"},
        "e2e": {"value": value, "unit": "guide-Gbp/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baselines(args, lens, guides, workdir):
    """CPU figures beside the GPU ones, all on this machine's cores: the
    reference's own CPU path (kind "reference") where it was built here, and
    the oracle's restatement (kind "port") as a second number.  Plain: the
    first 20 Mbp; batched: 8 of the 1,024 input files over the first 20 Mbp;
    PAM variety: the four 256-guide sets over the first 2 Mbp; served: 8 of
    the requests over the first 2 Mbp.  Rates are per base, extrapolated."""
    import random
    tools = cpu_binaries()
    threads = os.cpu_count() or 1
    kinds = [k for k in ("reference", "port") if tools[k]]
    total = sum(lens) + len(lens) - 1
    s20 = min(int(args.sample_mbp * 1e6), total)
    s2 = min(2_000_000, total)
    fa20 = write_genome(os.path.join(workdir, f"sample_{s20}.fa"), lens, limit=s20)
    fa2 = write_genome(os.path.join(workdir, f"sample_{s2}.fa"), lens, limit=s2)
    out = {"cores": threads, "primary": kinds[0]}
    for kind in kinds:
        b = tools[kind]
        dt, out_rows = cpu_run(b, input_text(fa20, guides), threads, workdir, "plain")
        res = {"plain": {"value": len(guides) * (s20 / 1e9) / dt, "seconds": dt, "rows": count_rows(out_rows),
                         "sample": f"first {s20} bp, 4 guides (extrapolated per base)"}}
        if not args.no_batched:
            texts = batched_jobs(genome_path=fa20)
            pick = random.Random(13).sample(range(len(texts)), 8)
            ts = [cpu_run(b, texts[j], threads, workdir, "batched")[0] for j in pick]
            res["batched"] = {"value": (s20 / 1e9) * len(ts) / sum(ts), "seconds": sum(ts),
                              "sample": f"input files {pick} of the 1,024 (one guide each), each alone over "
                                        f"the first {s20} bp (extrapolated per base and per input)"}
        if not args.no_pam_variety:
            ts = [cpu_run(b, t, threads, workdir, "pam")[0] for t in pam_variety_jobs(genome_path=fa2)]
            res["pam_variety"] = {"value": 1024 * (s2 / 1e9) / sum(ts), "seconds": sum(ts),
                                  "sample": f"the four 256-guide sets over the first {s2} bp (extrapolated per base)"}
        if not args.no_served:
            reqs = served_requests(n=args.served_requests, genome_path=fa2)
            pick = random.Random(17).sample(range(len(reqs)), min(8, len(reqs)))
            ts = [cpu_run(b, reqs[j][0], threads, workdir, "served")[0] for j in pick]
            g = sum(reqs[j][1] for j in pick)
            res["served"] = {"value": g * (s2 / 1e9) / sum(ts), "seconds": sum(ts),
                             "sample": f"requests {pick} ({g} guides), each alone over the first {s2} bp "
                                       f"(extrapolated per base)"}
        out[kind] = res
    return out


# ---------------------------------------------------------------- verification
def rows_of_records(rows, keep_names):
    """The rows (bytes, header lines dropped) whose chromosome is in keep_names,
    in their order."""
    keep = {n.encode() if isinstance(n, str) else n for n in keep_names}
    out = [l for l in rows.split(b"\n") if l and not l.startswith(b"#") and l.split(b"\t", 5)[4] in keep]
    return b"".join(l + b"\n" for l in out)


def compare_rows(gpu, ora):
    """{rows_compared, identical, first_difference} of two row texts (no headers)."""
    a, b = gpu.split(b"\n"), ora.split(b"\n")
    same = gpu == ora
    diff = None
    if not same:
        for i, (x, y) in enumerate(zip(a, b)):
            if x != y:
                diff = {"row": i, "gpu": x.decode(errors="replace")[:200], "oracle": y.decode(errors="replace")[:200]}
                break
        else:
            diff = {"row": min(len(a), len(b)), "gpu_rows": len(a), "oracle_rows": len(b)}
    return {"rows_compared": count_rows(ora), "gpu_rows": count_rows(gpu), "identical": same,
            "first_difference": diff}


def oracle_rows(oracle, text, threads, workdir, tag):
    """(seconds, the oracle's rows without the two header lines)."""
    dt, out = cpu_run(oracle, text, threads, workdir, tag)
    return dt, b"".join(l + b"\n" for l in out.split(b"\n") if l and not l.startswith(b"#"))


def run_verify(capture, lens, guides, names, workdir):
    """Byte comparison of the GPU rows captured from the timed legs against the
    oracle run on the same inputs (see the module docstring)."""
    import build_oracle
    oracle, _ = build_oracle.build(with_reference=False)
    threads = os.cpu_count() or 1
    res = {"oracle": "oracle/cof_oracle.cpp (CPU restatement, pinned to the reference's outputs)",
           "threads": threads}
    full = write_genome(os.path.join(workdir, "genome.2bit"), lens)
    if "plain" in capture:
        dt, ora = oracle_rows(oracle, input_text(full, guides), threads, workdir, "v_plain")
        res["plain"] = dict(compare_rows(capture["plain"], ora), oracle_s=round(dt, 1),
                            scope=f"whole genome: {len(lens)} records, {sum(lens) + len(lens) - 1} positions")
    os.remove(full)
    for leg, texts_of in (("batched", lambda path: batched_jobs(genome_path=path)),
                          ("pam_variety", lambda path: pam_variety_jobs(genome_path=path)),
                          ("served", lambda path: [t for t, _ in served_requests(n=capture.get("served_n", 0),
                                                                                  genome_path=path)])):
        cap = capture.get(leg)
        if not cap:
            continue
        k = cap["records"]
        path = write_genome(os.path.join(workdir, f"prefix{k}.2bit"), lens, records=k)
        texts = texts_of(path)
        items, t_all, ok = [], 0.0, True
        for j, gpu in cap["rows"].items():
            dt, ora = oracle_rows(oracle, texts[j], threads, workdir, f"v_{leg}")
            c = compare_rows(gpu, ora)
            items.append({"input": j, "rows_compared": c["rows_compared"], "identical": c["identical"],
                          "first_difference": c["first_difference"]})
            t_all += dt
            ok = ok and c["identical"]
        res[leg] = {"identical": ok, "rows_compared": sum(x["rows_compared"] for x in items), "inputs": items,
                    "oracle_s": round(t_all, 1),
                    "scope": f"rows on the first {k} records ({', '.join(names[:k])}: "
                             f"{sum(lens[:k]) + k - 1} positions) of the timed search"}
    res["identical"] = all(res[l]["identical"] for l in ("plain", "batched", "pam_variety", "served") if l in res)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--genome-gbp", type=float, default=3.1)
    ap.add_argument("--sample-mbp", type=float, default=20.0, help="CPU baseline sample (Mbp)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-search", choices=["plain", "batched", "pam_variety"], default=None,
                    help="profiling aid: warm up, then run ONE profiled search of that workload between "
                         "cudaProfilerStart/Stop (for ncu --profile-from-start off) and print its per-kernel "
                         "statistics as JSON instead of the benchmark line")
    ap.add_argument("--no-batched", action="store_true", help="skip the 1,024-guide batched comparison")
    ap.add_argument("--batched-steps", type=int, default=2)
    ap.add_argument("--plain-sample", type=int, default=32, help="plain searches timed for the comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served request stream")
    ap.add_argument("--no-pam-variety", action="store_true", help="skip the four 256-guide PAM sets")
    ap.add_argument("--comparer", default="auto", choices=["auto", "popcount", "bitsliced"],
                    help="comparer kernel for the plain search (default: bit-sliced where it fits)")
    ap.add_argument("--no-verify", action="store_true", help="skip the byte comparison with the oracle")
    ap.add_argument("--served-requests", type=int, default=200, help="requests per arrival rate")
    ap.add_argument("--served-rates", type=float, nargs="+", default=[1.0, 2.0, 5.0, 10.0, 20.0, 50.0, 100.0, 200.0])
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return
    if args.profile_search:
        profile_search(args)
        return

    import ctypes
    import numpy as np
    import torch
    P = pkg()
    P.build()
    torch.cuda.set_device(local)
    guides = make_guides()
    total_bp = args.genome_gbp * 1e9
    t0 = time.time()
    buf, names, starts, lens = build_genome(P, total_bp)
    n = len(buf)
    W = P.plane_words(n)
    # Planes packed straight into pinned host memory (the e2e source buffers).
    pinned = torch.empty(3 * W, dtype=torch.int32, pin_memory=True)
    planes = pinned.numpy().view(np.uint32)
    hi, lo, ot = planes[:W], planes[W:2 * W], planes[2 * W:]
    _, _, _, exc_pos, _ = P.pack_text(buf, out=(hi, lo, ot))
    assert exc_pos.size == 0  # the synthetic genome holds only A/C/G/T/N and ';'
    gen_s = time.time() - t0

    eng = P.CasOFFinder(local)
    eng.set_comparer({"auto": 0, "popcount": 1, "bitsliced": 2}[args.comparer])
    eng.readInputFile(input_text("synthetic", guides))
    info = eng.input_info()
    eng.load_genome_planes(hi, lo, ot, n, None, None, names, starts)
    h2d_bytes = 3 * W * 4 + sum(len(x) for x in names) + 8 * len(starts)

    # Warm-up (also sizes every device buffer).
    rows_len = 0
    for _ in range(args.warmup):
        addr, rows_len = eng.search_view()
    nh, nrows = eng.last_hit_count()
    schedule = eng.schedule().strip()

    # ---- per-kernel times (CUDA events around every launch): one profiled
    # search, outside the timed region
    eng.synchronize()
    eng.reset_stats()
    eng.set_profiling(True)
    eng.search_view()
    eng.set_profiling(False)
    stats = {k: eng.kernel_stats(k) for k in ("finder", "comparer", "format")}
    stages = {k: eng.kernel_stats(k)["ms"] for k in ("sort", "rows_to_host")}
    tests_stat = eng.kernel_stats("comparer.tests")

    # ---- value: genome resident in HBM (passes replayed as a CUDA graph)
    dist_barrier(world)
    eng.synchronize()
    with ClockSampler(local) as clk:
        eng.timer_start()
        for _ in range(args.steps):
            view = eng.search_view()
        ms = eng.timer_stop()
    capture = {"plain": ctypes.string_at(*view)}  # the rows of the last timed search
    ms_step = dist_max(ms / args.steps, world)
    gbp = sum(lens) / 1e9
    value = world * N_GUIDES * gbp / (ms_step / 1e3)

    # ---- e2e: host planes -> device, search, rows -> host, every step
    for _ in range(1):
        eng.search_planes_view(hi, lo, ot, n, None, None, names, starts)
    dist_barrier(world)
    eng.synchronize()
    eng.timer_start()
    for _ in range(args.steps):
        _, rows_len = eng.search_planes_view(hi, lo, ot, n, None, None, names, starts)
    e2e_ms = dist_max(eng.timer_stop() / args.steps, world)
    e2e_value = world * N_GUIDES * gbp / (e2e_ms / 1e3)
    # The same host -> device bytes copied alone (one copy of the pinned
    # planes, CUDA events): the floor under the e2e step.
    dev = torch.empty(3 * W, dtype=torch.int32, device=f"cuda:{local}")
    dev.copy_(pinned, non_blocking=True)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h2d = []
    for _ in range(3):
        ev0.record()
        dev.copy_(pinned, non_blocking=True)
        ev1.record()
        ev1.synchronize()
        h2d.append(ev0.elapsed_time(ev1))
    h2d_alone_ms = min(h2d)
    del dev

    # ---- roofline of the dominant kernel (comparer: integer pipes)
    rates = P.pipe_rates(local)
    d2h = P.d2h_rates(local)
    cmp = stats["comparer"]
    cinfo = eng.comparer_info()
    nw = 1 if info["pattern_len"] <= 32 else 2
    achieved = cmp["units"] / (cmp["ms"] * 1e-3) / 1e9 if cmp["ms"] else 0.0  # G base comparisons / s
    tests = tests_stat["units"]
    mean_nonN = cmp["units"] / tests if tests else 0.0  # base comparisons per variant test
    if cinfo["kind"] == "bit-sliced":
        # Full-adder tree: 2 LOP3 per (position, 32 candidates) = 1/16 LOP3 per base comparison.
        peak = rates["lop3"] * 16 / 1e9
        basis = (f"bit-sliced comparer ({cinfo['slots']} slots): 2 LOP3 per 32 base comparisons; measured LOP3 "
                 f"{rates['lop3'] / 1e12:.2f} T lane-ops/s")
    else:
        tests_per_s = min(rates["lop3"] / (4 * nw), rates["popc"] / nw)
        peak = tests_per_s * mean_nonN / 1e9
        basis = (f"popcount comparer: {4 * nw} LOP3 + {nw} POPC per variant test, {mean_nonN:.2f} base "
                 f"comparisons per test; measured LOP3 {rates['lop3'] / 1e12:.2f}, POPC {rates['popc'] / 1e12:.2f} "
                 f"T lane-ops/s")
    traffic = committed_traffic("comparer")
    issued = issued_roofline(eng, cmp, rates)
    # Finder bytes: 0.375 B of planes read per position scanned plus the 4 B
    # queue entry written per candidate; the profiled search runs each
    # finder launch alone, so its events time the kernel itself.
    fnd = stats["finder"]
    cands = eng.kernel_stats("finder.candidates")["units"]
    finder_bytes = fnd["units"] * 0.375 + cands * 4
    finder_gbs = finder_bytes / (fnd["ms"] * 1e-3) / 1e9 if fnd["ms"] else 0.0
    peaks = load_peaks()

    cpu = None
    workdir = tempfile.mkdtemp(prefix="cof_bench_")
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baselines(args, lens, guides, workdir)
        except Exception as e:  # the baseline is reported, never required
            cpu = {"failed": f"{e}"[:300]}

    # Kernels of ours per search (finder and comparer per segment; row
    # lengths and job bounds once; row writing in one launch per chunk, as
    # the profiled search counted them), times the timed searches.
    row_chunks = int(eng.kernel_stats("rows.chunks")["units"])
    launches = args.steps * int(stats["finder"]["launches"] + stats["comparer"]["launches"] +
                                (2 + row_chunks) * stats["format"]["launches"])
    batched = None if args.no_batched else run_batched(P, eng, lens, rates, args, capture)
    pam_variety = None if args.no_pam_variety else run_pam_variety(P, eng, lens, rates, args, capture)
    served = None if args.no_served else run_served(P, eng, lens, args, capture)
    cpu_main = None
    if cpu and "primary" in cpu:
        k = cpu["primary"]
        cpu_main = {"value": cpu[k]["plain"]["value"], "unit": "guide-Gbp/s", "cores": cpu["cores"], "kind": k,
                    "sample": cpu[k]["plain"]["sample"] + f" ({cpu[k]['plain']['rows']} rows, "
                                                          f"{cpu[k]['plain']['seconds']:.2f} s)"}
        if "port" in cpu and k != "port":
            cpu_main["port"] = {"value": cpu["port"]["plain"]["value"], "seconds": cpu["port"]["plain"]["seconds"]}
        for leg, obj in (("batched", batched), ("pam_variety", pam_variety), ("served", served)):
            if obj is not None and leg in cpu[k]:
                obj["cpu_baseline"] = dict(cpu[k][leg], unit="guide-Gbp/s", cores=cpu["cores"], kind=k)
                if "port" in cpu and k != "port" and leg in cpu["port"]:
                    obj["cpu_baseline"]["port"] = {"value": cpu["port"][leg]["value"]}
    elif cpu:
        cpu_main = {"value": None, "unit": "guide-Gbp/s", "cores": os.cpu_count(), "kind": "port",
                    "sample": cpu.get("failed")}
    verify = None
    if rank == 0 and not args.no_verify:
        eng.close()
        eng = None
        try:
            verify = run_verify(capture, lens, guides, names, workdir)
        except Exception as e:
            verify = {"identical": False, "failed": f"{e}"[:500]}
    shutil.rmtree(workdir, ignore_errors=True)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "guide-Gbp/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "genome_bp": n, "variants": info["variants"], "pattern_len": info["pattern_len"],
                       "hits": nh, "rows": nrows, "l2": "no flush: inputs (1.16 GB planes) exceed L2",
                       "genome_gen_s": round(gen_s, 1), "comparer_schedule": schedule},
            "e2e": {"value": e2e_value, "unit": "guide-Gbp/s", "h2d_bytes_per_step": h2d_bytes,
                    "d2h_bytes_per_step": rows_len + 16, "ms_per_step": e2e_ms,
                    "planes_h2d_alone_ms": h2d_alone_ms,
                    "planes_h2d_alone_gbs": 3 * W * 4 / (h2d_alone_ms * 1e-3) / 1e9,
                    "d2h_1gb_gbs": {"copy_engine": d2h["dma"] / 1e9, "sm_stores": d2h["sm"] / 1e9,
                                    "two_copy_engines": d2h["dma2"] / 1e9}},
            "roofline": {"bound": "int-pipe", "kernel": "comparer", "achieved": achieved, "peak": peak,
                         "unit": "G base-comparisons/s", "frac": achieved / peak if peak else None,
                         "traffic": traffic,
                         "peak_basis": basis, "base_comparisons_per_test": mean_nonN, "issued": issued,
                         "note": "the peak assumes every variant counted in full; the lane programs' update "
                                 "steps cost less per base comparison, so frac can pass 1 -- `issued` is the "
                                 "fraction of the LOP3 pipe the count phase itself occupies"},
            "roofline_finder": {"bound": "hbm", "achieved": finder_gbs, "peak": peaks.get("hbm_gbs"),
                                "unit": "GB/s", "frac": finder_gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs")
                                else None, "bytes_per_launch": finder_bytes / max(fnd["launches"], 1),
                                "us_per_launch": fnd["ms"] * 1e3 / max(fnd["launches"], 1),
                                "basis": "0.375 B per genome position (3 bit planes read) + 4 B per candidate "
                                         "(queue entry written); launches timed alone"},
            "kernel_ms_per_step": dict({k: v["ms"] for k, v in stats.items()}, **stages),
            "batched": batched,
            "pam_variety": pam_variety,
            "served": served,
            "cpu_baseline": cpu_main,
            "verify": verify,
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if eng is not None:
        eng.close()


VERIFY_BATCHED_JOBS, VERIFY_BATCHED_RECORDS = 8, 5  # 578 Mbp, 8 segment boundaries
VERIFY_PAM_SETS, VERIFY_PAM_RECORDS = (0, 3), 1      # NNGRRT and 5'-TTTV over chr1
VERIFY_SERVED_REQUESTS, VERIFY_SERVED_RECORDS = 2, 5


def run_batched(P, eng, lens, rates, args, capture=None):
    """The 1,024-guide mixed workload on the same resident genome: all 1,024
    input files in one batched search, against sequential plain searches (one
    input file at a time; a sample of them timed and scaled to 1,024)."""
    texts = batched_jobs()
    eng.batch_clear()
    for t in texts:
        eng.batch_add_input(t)
    info = eng.input_info()
    eng.search_view()  # warm-up (sizes every buffer, tunes the comparer)
    schedule = eng.schedule().strip()
    eng.synchronize()
    # Per-kernel times from one profiled search (events around every launch,
    # no CUDA graph); the value is timed without them.
    eng.reset_stats()
    eng.set_profiling(True)
    eng.search_view()
    eng.set_profiling(False)
    cmp = eng.kernel_stats("comparer")
    kernel_ms = {k: eng.kernel_stats(k)["ms"] for k in ("finder", "comparer", "sort", "format", "rows_to_host")}
    eng.synchronize()
    eng.timer_start()
    for _ in range(args.batched_steps):
        eng.search_view()
    ms = eng.timer_stop() / args.batched_steps
    hits, rows = eng.last_hit_count()
    gbp = sum(lens) / 1e9
    if capture is not None:  # rows of sampled jobs of the last timed search, on the leading records
        import random
        keep = [f"chr{i + 1}" for i in range(VERIFY_BATCHED_RECORDS)]
        pick = sorted(random.Random(11).sample(range(len(texts)), VERIFY_BATCHED_JOBS))
        capture["batched"] = {"records": VERIFY_BATCHED_RECORDS,
                              "rows": {j: rows_of_records(eng.job_rows(j), keep) for j in pick}}
    # Sequential plain searches of the same input files.
    k = args.plain_sample
    eng.readInputFile(texts[0])
    eng.search_view()
    eng.synchronize()
    eng.timer_start()
    for t in texts[:k]:
        eng.readInputFile(t)
        eng.search_view()
    plain_ms = eng.timer_stop() / k
    # Where a plain input's time goes: setup (parse, table upload, the
    # autotuner's timed trial launches, CUDA-graph capture: the first search
    # of an input minus a repeat) and the search itself (the repeat), with the
    # autotuner on (the default) and off.
    split = {}
    for tune in (True, False):
        eng.set_autotune(tune)
        setup, search = [], []
        for t in texts[:k]:
            eng.synchronize()
            t0 = time.perf_counter()
            eng.readInputFile(t)
            eng.search_view()
            t1 = time.perf_counter()
            eng.search_view()
            t2 = time.perf_counter()
            search.append((t2 - t1) * 1e3)
            setup.append(max(0.0, (t1 - t0) * 1e3 - search[-1]))
        split["autotune_on" if tune else "autotune_off"] = {
            "setup_ms": statistics.fmean(setup), "search_ms": statistics.fmean(search),
            "speedup_vs_plain_search_only": statistics.fmean(search) * len(texts) / ms}
    eng.set_autotune(True)
    achieved = cmp["units"] / (cmp["ms"] * 1e-3) / 1e9 if cmp["ms"] else 0.0
    peak = rates["lop3"] * 16 / 1e9
    return {
        "workload": "1,024 single-guide input files: spacer 20-24 (2% IUPAC), PAM NGG/NRG, mm 3-6, DNA bulge 0-2, "
                    "RNA bulge 0-1, on the same 3.1 Gbp genome",
        "value": len(texts) * gbp / (ms / 1e3), "unit": "guide-Gbp/s", "ms_per_step": ms,
        "steps": args.batched_steps, "variants": info["variants"], "hits": hits, "rows": rows,
        "plain_value": gbp / (plain_ms / 1e3), "plain_ms_per_input": plain_ms, "plain_sample_inputs": k,
        "plain_setup_ms": split["autotune_on"]["setup_ms"], "plain_search_ms": split["autotune_on"]["search_ms"],
        "plain_split": split,
        "speedup_vs_plain": (plain_ms * len(texts)) / ms, "kernel_ms_profiled": kernel_ms,
        "comparer_schedule": schedule,
        "comparer_roofline": {"achieved": achieved, "peak": peak, "unit": "G base-comparisons/s",
                              "frac": achieved / peak if peak else None,
                              "issued": issued_roofline(eng, cmp, rates)},
    }


def run_pam_variety(P, eng, lens, rates, args, capture=None):
    """The four 256-guide PAM sets in one batched search of the resident
    genome, against the four sets searched one after another."""
    texts = pam_variety_jobs()
    eng.batch_clear()
    for t in texts:
        eng.batch_add_input(t)
    info = eng.input_info()
    eng.search_view()  # warm-up (tunes the comparer)
    schedule = eng.schedule().strip()
    eng.synchronize()
    eng.reset_stats()
    eng.set_profiling(True)
    eng.search_view()
    eng.set_profiling(False)
    cmp = eng.kernel_stats("comparer")
    kernel_ms = {k: eng.kernel_stats(k)["ms"] for k in ("finder", "comparer", "format")}
    eng.timer_start()
    for _ in range(args.batched_steps):
        eng.search_view()
    ms = eng.timer_stop() / args.batched_steps
    hits, rows = eng.last_hit_count()
    gbp = sum(lens) / 1e9
    if capture is not None:
        keep = [f"chr{i + 1}" for i in range(VERIFY_PAM_RECORDS)]
        capture["pam_variety"] = {"records": VERIFY_PAM_RECORDS,
                                  "rows": {j: rows_of_records(eng.job_rows(j), keep) for j in VERIFY_PAM_SETS}}
    seq_ms = 0.0
    for t in texts:
        eng.readInputFile(t)
        eng.search_view()
        eng.synchronize()
        eng.timer_start()
        eng.search_view()
        seq_ms += eng.timer_stop()
    guides = 256 * len(texts)
    achieved = cmp["units"] / (cmp["ms"] * 1e-3) / 1e9 if cmp["ms"] else 0.0
    peak = rates["lop3"] * 16 / 1e9
    return {
        "workload": "4 input files x 256 guides: NNGRRT/21-nt, NNNNGMTT/24-nt, NNAGAAW/20-nt, 5'-TTTV/23-nt spacers, "
                    "mm 4, DNA bulge 1, RNA bulge 1, on the same 3.1 Gbp genome",
        "value": guides * gbp / (ms / 1e3), "unit": "guide-Gbp/s", "ms_per_step": ms, "steps": args.batched_steps,
        "variants": info["variants"], "hits": hits, "rows": rows,
        "sequential_value": guides * gbp / (seq_ms / 1e3), "sequential_ms": seq_ms,
        "speedup_vs_sequential": seq_ms / ms, "kernel_ms_profiled": kernel_ms, "comparer_schedule": schedule,
        "comparer_roofline": {"achieved": achieved, "peak": peak, "unit": "G base-comparisons/s",
                              "frac": achieved / peak if peak else None,
                              "issued": issued_roofline(eng, cmp, rates)},
    }


def profile_search(args):
    """One profiled search of a workload on a genome of --genome-gbp, after
    warm-up searches, between cudaProfilerStart and cudaProfilerStop, so that
    `ncu --profile-from-start off` captures exactly that search's launches.
    Prints the engine's per-kernel statistics (events, algorithmic units,
    the comparer's LOP3 op model) as one JSON line."""
    import numpy as np
    import torch
    P = pkg()
    P.build()
    buf, names, starts, lens = build_genome(P, args.genome_gbp * 1e9)
    n = len(buf)
    W = P.plane_words(n)
    hi, lo, ot = (np.empty(W, np.uint32) for _ in range(3))
    P.pack_text(buf, out=(hi, lo, ot))
    eng = P.CasOFFinder(0)
    if args.profile_search == "plain":
        eng.readInputFile(input_text("synthetic", make_guides()))
    else:
        eng.batch_clear()
        for t in (batched_jobs() if args.profile_search == "batched" else pam_variety_jobs()):
            eng.batch_add_input(t)
    eng.load_genome_planes(hi, lo, ot, n, None, None, names, starts)
    for _ in range(2):
        eng.search_view()
    eng.synchronize()
    eng.reset_stats()
    eng.set_profiling(True)
    torch.cuda.profiler.start()
    eng.search_view()
    eng.synchronize()
    torch.cuda.profiler.stop()
    eng.set_profiling(False)
    out = {k: eng.kernel_stats(k) for k in ("finder", "finder.candidates", "comparer", "comparer.tests",
                                            "comparer.lop3", "format")}
    out.update(workload=args.profile_search, genome_bp=n, schedule=eng.schedule().strip())
    print(json.dumps(out), flush=True)
    eng.close()


def issued_roofline(eng, cmp, rates):
    """The bit-sliced comparer against the LOP3 pipe by the instructions it
    issues: the engine's op model counts, per launch, the lane LOP3
    instructions of the count phase (full count, bias, update steps, votes;
    ceil(candidates / 64) pairs x 32 lanes x chunks x the per-lane count of the
    group's slots and program length), and this divides them by the comparer's
    time and the measured LOP3 rate.  Unlike the base-comparison figure it
    does not credit the lane programs for the work their steps avoid."""
    ops = eng.kernel_stats("comparer.lop3")["units"]
    if not ops or not cmp["ms"]:
        return None
    achieved = ops / (cmp["ms"] * 1e-3)
    return {"lop3_lane_ops": ops, "achieved": achieved / 1e12, "peak": rates["lop3"] / 1e12,
            "unit": "T lane-LOP3/s", "frac": achieved / rates["lop3"],
            "model": "count phase only (the table build's transposes and class words are not counted)"}


def committed_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(path)).get(kernel)
    except (OSError, ValueError):
        return None


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "fallback": True}


if __name__ == "__main__":
    main()
