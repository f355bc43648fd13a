#!/usr/bin/env python3
"""Generates the golden fixtures under tests/golden/<case>/ from the reference.

Each case directory holds a small seeded genome (FASTA or 2BIT), `input.txt`
(line 1 = the genome file name relative to the case directory) and
`expected.tsv`: the output of the reference Cas-OFFinder 3.0.0 itself, built
from its own sources by oracle/build_ref.py and run with device C and one
OpenMP thread (so rows come in the reference's sequential order).  Cases with
--summary also keep `expected_summary.txt`; cases the reference rejects keep
`expected_error.txt` (its exit code and message).  `mismatch_table.bin` is
the reference kernel's IUPAC mismatch predicate for all 256 x 256 byte pairs
(oracle/ref_shim/ref_predicate.cpp runs comparer_cpu on every pair).

Run (needs the reference checkout): python tests/golden/make_golden.py
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import cases  # noqa: E402
import build_ref  # noqa: E402

NGG = "N" * 21 + "GG"
NRG = "N" * 21 + "RG"

# name -> make_case keyword arguments (+ "summary": bool, "error": bool)
CASES = {
    "ngg_fasta": dict(seed=11, lens=[60000, 40000], pattern=NGG, mm=4, per_guide=25),
    "nrg_bulge_2bit": dict(seed=12, lens=[50000, 30000, 20000], fmt="2bit", pattern=NRG, dna=2, rna=1, mm=5,
                           per_guide=25, n_frac=0.05),
    "pam5_tttv": dict(seed=13, lens=[70000], pattern="TTTV" + "N" * 23, dna=1, rna=1, mm=4, per_guide=25),
    "iupac_nngrrt": dict(seed=14, lens=[40000, 30000], pattern="N" * 21 + "NNGRRT", mm=[3, 4, 5], per_guide=20,
                         iupac_frac=0.1, with_ids=True, sprinkle_chars="RYKMWSBDHVnacgtX*-"),
    "dup_guides_dna2": dict(seed=15, lens=[50000], pattern=NGG, dna=2, rna=1, mm=[4, 2], per_guide=20,
                            guides=["GGCCGACCTGTCGCTGACGCNNN", "AAAACCTGTCGCTGACGCCCNNN",
                                    "GGCCGACCTGTCGCTGACGCNNN", "GGGGGGGCTGTCGCTGAAAANNN"]),
    "crlf_record_edges": dict(seed=16, lens=[10, 0, 30000, 22, 25000], pattern=NGG, mm=4, per_guide=25, crlf=True,
                              n_frac=0.0),
    "allN_talen_long": dict(seed=17, lens=[6000, 3000], pattern="N" * 52, mm=[10, 12], per_guide=6, n_frac=0.0,
                            guides=["TTCTGGAGGTGCCTGAGGCCNNNNNNNNNNNNGAGGCCACCTTTCCAGTCCA",
                                    "TGGCCAATGTGACGCTGACGNNNNNNNNNNNNCTGGAGACTCCAGACTTCCA"]),
    "nnnngmtt_33": dict(seed=18, lens=[60000], pattern="N" * 24 + "NNNNGMTT", dna=1, rna=1, mm=5, per_guide=25),
    "summary_nag": dict(seed=19, lens=[40000, 40000], pattern="N" * 20 + "NAG", dna=1, rna=1, mm=4, per_guide=20,
                        with_ids=True, summary=True),
    "threshold_wraps": dict(seed=20, lens=[2500], pattern="N" * 21 + "GG", mm=-1, per_guide=2, n_frac=0.0,
                            n_guides=1),
    "genome_shorter_than_pattern": dict(seed=21, lens=[15], pattern=NGG, mm=4, per_guide=0, n_frac=0.0),
    "malformed_token_count": dict(seed=22, lens=[1000], pattern=NGG, mm=4, per_guide=0,
                                  extra_lines="ACGTACGTACGTACGTACGTNNN 3 id 9\n", error=True),
}


def rel_input(ipath, gname):
    lines = open(ipath).read().split("\n")
    lines[0] = gname
    return "\n".join(lines)


def main():
    ref = build_ref.build()
    if not ref:
        sys.exit("reference checkout not found: golden fixtures need the reference itself")
    manifest = {}
    for name, spec in CASES.items():
        spec = dict(spec)
        want_summary = spec.pop("summary", False)
        want_error = spec.pop("error", False)
        out_dir = os.path.join(HERE, name)
        if os.path.isdir(out_dir):
            shutil.rmtree(out_dir)
        os.makedirs(out_dir)
        with tempfile.TemporaryDirectory() as tmp:
            ipath, gpath = cases.make_case(tmp, **spec)
            gname = "genome" + os.path.splitext(gpath)[1]
            shutil.copy(gpath, os.path.join(out_dir, gname))
            with open(os.path.join(out_dir, "input.txt"), "w") as f:
                f.write(rel_input(ipath, gname))
            run_in = os.path.join(tmp, "run_input.txt")
            with open(run_in, "w") as f:
                f.write(rel_input(ipath, os.path.join(out_dir, gname)))
            out = os.path.join(tmp, "out.tsv")
            summ = os.path.join(tmp, "summary.txt") if want_summary else None
            r = cases.run_cli(ref, run_in, out, threads=1, device="C", summary=summ)
            if want_error:
                assert r.returncode != 0, name
                with open(os.path.join(out_dir, "expected_error.txt"), "w") as f:
                    msg = [l for l in r.stderr.decode().splitlines() if l.startswith("Critical error!")]
                    f.write(f"{r.returncode}\n{msg[0] if msg else ''}\n")
                manifest[name] = {"error": True}
                continue
            assert r.returncode == 0, (name, r.stderr.decode())
            shutil.copy(out, os.path.join(out_dir, "expected.tsv"))
            if summ:
                shutil.copy(summ, os.path.join(out_dir, "expected_summary.txt"))
            rows = len(cases.rows_of(open(out, "rb").read()))
            manifest[name] = {"rows": rows, "summary": bool(summ)}
            print(f"{name}: {rows} rows")
    # The reference kernel's mismatch predicate over all 256 x 256 byte pairs.
    pred = os.path.join(os.path.dirname(ref), "ref-predicate")
    subprocess.run([pred, os.path.join(HERE, "mismatch_table.bin")], check=True)
    manifest["mismatch_table.bin"] = {"bytes": 65536, "source": "comparer_cpu of the reference"}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
