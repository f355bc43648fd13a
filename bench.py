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
          (cof_search_planes: the upload of segment s+1 overlaps the scan of
          segment s), and copies the rows back.
The genome planes (1.16 GB) are larger than L2, so no flush is needed between
steps.  Timing: CUDA events on the engine's stream (cof_timer_start/stop),
after warm-up steps, max over ranks.  Under torchrun each rank runs an
independent replica on its own GPU (weak scaling; the search has no
cross-GPU exchange).

--impl reference times the reference algorithm on the host CPU cores instead:
the reference binary built from its sources when it runs here, else the
oracle's CPU restatement, on a bounded prefix of the same genome.
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


def run_served(P, eng, lens, args):
    """Served mode: the same requests arriving as a Poisson stream at several
    rates; p50/p99 latency (submit to rows in host memory) and guide-Gbp/s,
    against the plain path run once per request."""
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
    out = {"workload": f"{len(reqs)} requests, 1-512 guides each (log-uniform; {guides} guides), PAM NGG/NRG/"
                       "NNGRRT/TTTV, mm 2-6, DNA/RNA bulge 0-2, on the same 3.1 Gbp genome",
           "plain_value": guides * gbp / (sum(plain_ms) / 1e3), "unit": "guide-Gbp/s",
           "plain_latency_ms": {"p50": statistics.median(plain_ms), "max": max(plain_ms)}, "rates": []}
    for rate in args.served_rates:
        rng = random.Random(int(rate * 1000))
        lat, tickets = [None] * len(reqs), [None] * len(reqs)
        with P.Server(eng) as srv:
            t0 = time.perf_counter()

            # Each arrival is submitted from its own thread, as concurrent
            # callers would (submit parses the input file on the caller's
            # thread).
            def submit(j, at):
                d = at - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                tickets[j] = srv.submit(reqs[j][0])

            threads, at = [], t0
            for j in range(len(reqs)):
                at += rng.expovariate(rate)
                threads.append(threading.Thread(target=submit, args=(j, at)))
                threads[-1].start()
            for th in threads:
                th.join()
            for j in range(len(reqs)):
                _, _, lat[j] = srv.wait_view(tickets[j])  # rows left in the server's pinned buffer
            span = time.perf_counter() - t0
            for j in range(len(reqs)):
                srv.release(tickets[j])
            st = srv.stats()
        lat_sorted = sorted(lat)
        p99 = lat_sorted[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]
        out["rates"].append({"arrivals_per_s": rate, "p50_ms": statistics.median(lat), "p99_ms": p99,
                             "value": guides * gbp / span, "makespan_s": span, "max_active": st["max_active"],
                             "ring_steps": st["steps"]})
    out["value"] = max(r["value"] for r in out["rates"])
    out["speedup_vs_plain"] = out["value"] / out["plain_value"]
    return out


def input_text(genome_path, guides):
    return f"{genome_path}\n{PATTERN} {DNA} {RNA}\n" + "".join(f"{g} {MM}\n" for g in guides)


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
        P.lib().cofx_synth_record(seed, r, ln, 0.41, 0.10, 100000, 0.05, 1000, 100000, base + pos)
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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


def cpu_sample_run(binary, genome_buf, names, starts, sample_bp, guides, threads, workdir):
    """Runs the CPU implementation on the first `sample_bp` positions of the
    genome (as FASTA); returns (seconds, rows)."""
    fa = os.path.join(workdir, "sample.fa")
    if not os.path.exists(fa):
        end = min(len(genome_buf), sample_bp)
        P = pkg()
        recs, nm = [], []
        for i, s in enumerate(starts):
            e = (starts[i + 1] - 1) if i + 1 < len(starts) else len(genome_buf)
            if s >= end:
                break
            recs.append(bytes(genome_buf[s:min(e, end)]))
            nm.append(names[i])
        P.write_fasta(fa, nm, recs)
    inp = os.path.join(workdir, "sample_input.txt")
    with open(inp, "w") as f:
        f.write(input_text(fa, guides))
    out = os.path.join(workdir, "sample_out.tsv")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    t0 = time.perf_counter()
    r = subprocess.run([binary, inp, "C", out], env=env, capture_output=True)
    dt = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(r.stderr.decode()[-2000:])
    rows = sum(1 for l in open(out, "rb") if not l.startswith(b"#"))
    return dt, rows


def cpu_binary():
    """(path, kind): the reference built from its sources if it runs here, else the oracle port."""
    import build_oracle
    port, _ = build_oracle.build(with_reference=False)
    ref_path = os.path.join(ROOT, "oracle", "_ref", "cas-offinder-ref")  # prebuilt by build(), if at all
    for cand, kind in ((ref_path, "reference"), (port, "port")):
        if cand and os.path.exists(cand):
            try:
                r = subprocess.run([cand], capture_output=True, timeout=30)
                if r.returncode == 0:
                    return cand, kind
            except OSError:
                continue
    raise RuntimeError("no CPU implementation available")


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    P = pkg()
    P.build()
    binary, kind = cpu_binary()
    guides = make_guides()
    sample_bp = int(args.sample_mbp * 1e6)
    buf, names, starts, _ = build_genome(P, args.genome_gbp * 1e9, prefix_bp=sample_bp)
    threads = os.cpu_count() or 1
    times = []
    with tempfile.TemporaryDirectory() as tmp:
        for i in range(args.warmup + args.steps):
            dt, rows = cpu_sample_run(binary, buf, names, starts, sample_bp, guides, threads, tmp)
            if i >= args.warmup:
                times.append(dt)
    total = sum(times)
    gbp = min(len(buf), sample_bp) / 1e9
    value = N_GUIDES * gbp * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "guide-Gbp/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_bp": min(len(buf), sample_bp)},
        "cpu_baseline": {"value": value, "unit": "guide-Gbp/s", "cores": threads, "kind": kind,
                         "sample": f"first {min(len(buf), sample_bp)} bp of the same genome and input "
                                   f"({rows} rows)"},
        "e2e": {"value": value, "unit": "guide-Gbp/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--genome-gbp", type=float, default=3.1)
    ap.add_argument("--sample-mbp", type=float, default=20.0, help="CPU baseline sample (Mbp)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 1,024-guide batched comparison")
    ap.add_argument("--batched-steps", type=int, default=2)
    ap.add_argument("--plain-sample", type=int, default=32, help="plain searches timed for the comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served request stream")
    ap.add_argument("--no-pam-variety", action="store_true", help="skip the four 256-guide PAM sets")
    ap.add_argument("--comparer", default="auto", choices=["auto", "popcount", "bitsliced"],
                    help="comparer kernel for the plain search (default: bit-sliced where it fits)")
    ap.add_argument("--served-requests", type=int, default=12)
    ap.add_argument("--served-rates", type=float, nargs="+", default=[1.0, 2.0, 5.0, 10.0, 20.0, 50.0, 100.0, 200.0])
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

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
    tests_stat = eng.kernel_stats("comparer.tests")

    # ---- value: genome resident in HBM (passes replayed as a CUDA graph)
    dist_barrier(world)
    eng.synchronize()
    with ClockSampler(local) as clk:
        eng.timer_start()
        for _ in range(args.steps):
            eng.search_view()
        ms = eng.timer_stop()
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

    # ---- roofline of the dominant kernel (comparer: integer pipes)
    rates = P.pipe_rates(local)
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
    # Finder bytes: 0.375 B of planes read per position scanned plus the 4 B
    # queue entry written per candidate; the profiled search runs each
    # finder launch alone, so its events time the kernel itself.
    fnd = stats["finder"]
    cands = eng.kernel_stats("finder.candidates")["units"]
    finder_bytes = fnd["units"] * 0.375 + cands * 4
    finder_gbs = finder_bytes / (fnd["ms"] * 1e-3) / 1e9 if fnd["ms"] else 0.0
    peaks = load_peaks()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            binary, kind = cpu_binary()
            with tempfile.TemporaryDirectory() as tmp:
                sample_bp = int(args.sample_mbp * 1e6)
                threads = os.cpu_count() or 1
                dt, srows = cpu_sample_run(binary, buf, names, starts, sample_bp, guides, threads, tmp)
                cpu = {"value": N_GUIDES * (sample_bp / 1e9) / dt, "unit": "guide-Gbp/s", "cores": threads,
                       "kind": kind, "sample": f"first {sample_bp} bp of the same genome and input "
                                               f"({srows} rows, {dt:.2f} s)"}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "guide-Gbp/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"[:300]}

    # Kernels of ours per search (finder and comparer per segment; row
    # lengths and job bounds once; row writing in one launch per chunk of
    # max(2^16, ceil(hits / 8)) hits), times the timed searches.
    chunk_hits = max(1 << 16, -(-nh // 8))
    row_chunks = -(-nh // chunk_hits) if nh else 0
    launches = args.steps * int(stats["finder"]["launches"] + stats["comparer"]["launches"] +
                                (2 + row_chunks) * stats["format"]["launches"])
    batched = None if args.no_batched else run_batched(P, eng, lens, rates, args)
    pam_variety = None if args.no_pam_variety else run_pam_variety(P, eng, lens, rates, args)
    served = None if args.no_served else run_served(P, eng, lens, args)
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
                    "d2h_bytes_per_step": rows_len + 16, "ms_per_step": e2e_ms},
            "roofline": {"bound": "int-pipe", "kernel": "comparer", "achieved": achieved, "peak": peak,
                         "unit": "G base-comparisons/s", "frac": achieved / peak if peak else None,
                         "traffic": traffic,
                         "peak_basis": basis, "base_comparisons_per_test": mean_nonN},
            "roofline_finder": {"bound": "hbm", "achieved": finder_gbs, "peak": peaks.get("hbm_gbs"),
                                "unit": "GB/s", "frac": finder_gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs")
                                else None, "bytes_per_launch": finder_bytes / max(fnd["launches"], 1),
                                "us_per_launch": fnd["ms"] * 1e3 / max(fnd["launches"], 1),
                                "basis": "0.375 B per genome position (3 bit planes read) + 4 B per candidate "
                                         "(queue entry written); launches timed alone"},
            "kernel_ms_per_step": {k: v["ms"] for k, v in stats.items()},
            "batched": batched,
            "pam_variety": pam_variety,
            "served": served,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    eng.close()


def run_batched(P, eng, lens, rates, args):
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
    kernel_ms = {k: eng.kernel_stats(k)["ms"] for k in ("finder", "comparer", "format")}
    eng.synchronize()
    eng.timer_start()
    for _ in range(args.batched_steps):
        eng.search_view()
    ms = eng.timer_stop() / args.batched_steps
    hits, rows = eng.last_hit_count()
    gbp = sum(lens) / 1e9
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
    achieved = cmp["units"] / (cmp["ms"] * 1e-3) / 1e9 if cmp["ms"] else 0.0
    peak = rates["lop3"] * 16 / 1e9
    return {
        "workload": "1,024 single-guide input files: spacer 20-24 (2% IUPAC), PAM NGG/NRG, mm 3-6, DNA bulge 0-2, "
                    "RNA bulge 0-1, on the same 3.1 Gbp genome",
        "value": len(texts) * gbp / (ms / 1e3), "unit": "guide-Gbp/s", "ms_per_step": ms,
        "steps": args.batched_steps, "variants": info["variants"], "hits": hits, "rows": rows,
        "plain_value": gbp / (plain_ms / 1e3), "plain_ms_per_input": plain_ms, "plain_sample_inputs": k,
        "speedup_vs_plain": (plain_ms * len(texts)) / ms, "kernel_ms_profiled": kernel_ms,
        "comparer_schedule": schedule,
        "comparer_roofline": {"achieved": achieved, "peak": peak, "unit": "G base-comparisons/s",
                              "frac": achieved / peak if peak else None},
    }


def run_pam_variety(P, eng, lens, rates, args):
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
                              "frac": achieved / peak if peak else None},
    }


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
