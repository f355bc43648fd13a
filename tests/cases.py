"""Seeded synthetic search cases for the parity tests.

A case is a genome file (FASTA or 2BIT) plus an input file.  To keep the
parity checks non-vacuous, guide-derived sites are planted into the random
genome: the guide's non-N bases with the pattern's PAM filled in, a few random
substitutions and sometimes a DNA or RNA bulge, on either strand, some of them
next to record ends.
"""
import os
import random
import subprocess

import numpy as np

from pkgload import pkg

IUPAC = "ACGTRYKMWSHBVDN"
COMP = str.maketrans("ACGTRYKMWSHBVDN", "TGCAYRMKWSDVBHN")

# A concrete base that satisfies each pattern byte.
FILL = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "K": "GT", "M": "AC", "W": "AT", "S": "CG",
        "H": "ACT", "B": "CGT", "V": "ACG", "D": "AGT", "N": "ACGT"}


def revcomp(s):
    return s.translate(COMP)[::-1]


def random_guides(rng, n, spacer, pam, pam5=False, iupac_frac=0.0):
    """n guides: `spacer` random bases (a fraction `iupac_frac` degenerate) and
    N over the PAM positions, in the input file's orientation."""
    out = []
    for _ in range(n):
        sp = "".join(rng.choice("ACGT") if rng.random() >= iupac_frac else rng.choice("RYKMWSHBVD")
                      for _ in range(spacer))
        out.append(("N" * len(pam) + sp) if pam5 else (sp + "N" * len(pam)))
    return out


def plant_sites(rng, seqs, pattern, guides, per_guide, max_sub, dna=0, rna=0, near_ends=True):
    """Write mutated copies of guide sites into `seqs` (list of bytearray)."""
    for g in guides:
        for _ in range(per_guide):
            # Concrete site: guide bases where not N, else a base satisfying the
            # pattern byte (the raw pattern line and the guides have one length).
            site = [rng.choice(FILL.get(c if c != "N" else p, "ACGT")) for p, c in zip(pattern, g)]
            site = list("".join(site))
            for _ in range(rng.randint(0, max_sub)):
                k = rng.randrange(len(site))
                site[k] = rng.choice("ACGT")
            kind = rng.random()
            if dna and kind < 0.3:
                k = rng.randrange(1, len(site))
                site[k:k] = [rng.choice("ACGT") for _ in range(rng.randint(1, dna))]
            elif rna and kind < 0.6:
                k = rng.randrange(1, len(site) - rna)
                del site[k:k + rng.randint(1, rna)]
            s = "".join(site)
            if rng.random() < 0.5:
                s = revcomp(s)
            r = rng.randrange(len(seqs))
            L = len(seqs[r])
            if L < len(s) + 2:
                continue
            if near_ends and rng.random() < 0.1:
                at = rng.choice([0, L - len(s), rng.randrange(0, 40) if L > 80 else 0])
            else:
                at = rng.randrange(0, L - len(s))
            seqs[r][at:at + len(s)] = s.encode()


def sprinkle(rng, seqs, chars, count):
    """Overwrite `count` random positions with bytes from `chars` (IUPAC, lower case, ...)."""
    for _ in range(count):
        r = rng.randrange(len(seqs))
        if len(seqs[r]):
            seqs[r][rng.randrange(len(seqs[r]))] = ord(rng.choice(chars))


def write_genome(path, fmt, names, seqs, crlf=False, width=60):
    P = pkg()
    if fmt == "2bit":
        P.write_twobit(path, names, seqs)
    else:
        P.write_fasta(path, names, seqs, width=width)
        if crlf:
            data = open(path, "rb").read().replace(b"\n", b"\r\n")
            open(path, "wb").write(data)


def make_case(workdir, seed, lens, fmt="fasta", pattern="NNNNNNNNNNNNNNNNNNNNNGG", dna=0, rna=0, n_guides=4,
              mm=4, per_guide=30, max_sub=None, with_ids=False, n_frac=0.01, iupac_frac=0.0, sprinkle_chars=None,
              crlf=False, guides=None, gc_drift=0.0, extra_lines=""):
    """Builds one case under `workdir`; returns (input_path, genome_path)."""
    rng = random.Random(seed)
    P = pkg()
    seqs = [P.synth_record(seed, r, n, gc=0.41, gc_drift=gc_drift, n_frac=n_frac, n_run_min=50, n_run_max=500)
            for r, n in enumerate(lens)]
    pam5 = pattern[0] != "N"
    core = pattern.lstrip("N") if not pam5 else pattern.rstrip("N")
    spacer = len(pattern) - len(core)
    if guides is None:
        guides = random_guides(rng, n_guides, spacer, core, pam5, iupac_frac)
    top = mm if isinstance(mm, int) else max(mm)
    plant_sites(rng, seqs, pattern, guides, per_guide, max(0, min(top + 1, 8)) if max_sub is None else max_sub, dna, rna)
    if sprinkle_chars:
        sprinkle(rng, seqs, sprinkle_chars, max(1, sum(lens) // 2000))
    names = [f"chr{r + 1}" for r in range(len(lens))]
    gpath = os.path.join(workdir, f"genome_{seed}.{'2bit' if fmt == '2bit' else 'fa'}")
    write_genome(gpath, fmt, names, seqs, crlf=crlf)
    lines = [gpath, pattern + (f" {dna} {rna}" if (dna or rna) else "")]
    for i, g in enumerate(guides):
        m = mm if isinstance(mm, int) else mm[i % len(mm)]
        lines.append(f"{g} {m}" + (f" g{i}" if with_ids else ""))
    ipath = os.path.join(workdir, f"input_{seed}.txt")
    with open(ipath, "w") as f:
        f.write("\n".join(lines) + "\n" + extra_lines)
    return ipath, gpath


def run_cli(binary, input_path, out_path, threads=1, device="C", summary=None, timeout=600):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    cmd = [binary, input_path, device, out_path]
    if summary:
        cmd = [binary, "--summary", summary, input_path, device, out_path]
    r = subprocess.run(cmd, env=env, capture_output=True, timeout=timeout)
    return r


def canonical(text: bytes):
    """Header lines kept in place, data rows sorted (multiset order)."""
    lines = text.split(b"\n")
    head = [l for l in lines if l.startswith(b"#")]
    rows = sorted(l for l in lines if l and not l.startswith(b"#"))
    return head, rows


def rows_of(text: bytes):
    return [l for l in text.split(b"\n") if l and not l.startswith(b"#")]


def np_seed(seed):
    return np.random.default_rng(seed)


IUPAC_SETS = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "K": "GT", "M": "AC", "S": "CG",
              "W": "AT", "B": "CGT", "D": "AGT", "H": "ACT", "V": "ACG", "N": "ACGT"}


def shown_mismatch(p, g):
    """Whether the reference lower-cases genome base g under pattern byte p
    (cas-offinder.cpp:299-317): a non-ACGT genome byte only under a concrete
    base, otherwise when g is outside p's IUPAC set."""
    if p == "N" or p not in IUPAC_SETS:
        return False
    if g not in "ACGT":
        return p in "ACGT"
    return g not in IUPAC_SETS[p]


def row_problems(row: str):
    """Checks of one output row that need no genome: lower case exactly where
    an aligned crRNA letter mismatches, and the lower-case count equals the
    mismatch column.  A DNA-bulge base is compared with the pattern base the
    crRNA column shows as '-', so it counts without an aligned letter; a '-'
    strand RNA-bulge row's columns end short of the compared window
    (cas-offinder.cpp:441-442), so there the count is only a lower bound.
    Returns a list of problems (empty when the row passes)."""
    f = row.split("\t")
    crrna, dna, strand, mm = f[2], f[3], f[6], int(f[7])
    bases = [c for c in dna if c != "-"]
    crb = [c for c, d in zip(crrna, dna) if d != "-"]
    out = []
    for i, (p, g) in enumerate(zip(crb, bases)):
        if p != "-" and g.islower() != shown_mismatch(p.upper(), g.upper()):
            out.append(f"case of base {i}")
    low = sum(c.islower() for c in bases)
    if f[1] == "RNA" and strand == "-":
        if low > mm:
            out.append(f"{low} lower-case > {mm}")
    elif low != mm:
        out.append(f"{low} lower-case != {mm}")
    return out


# ---------------------------------------------------------------- kernel restatement
def mismatch_table():
    """The reference kernel's mismatch predicate as a 256 x 256 table
    [pattern byte][genome byte] (golden fixture dumped from cas-offinder.cl)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mismatch_table.bin")
    return np.fromfile(path, np.uint8).reshape(256, 256)


def _revcomp_bytes(s):
    return bytes(s[::-1]).translate(bytes.maketrans(b"ACGTRYKMHDBV", b"TGCAYRMKDHVB"))


def _mismatch_counts(M, g, s, starts):
    """Mismatches of pattern string `s` against g[i:i+len(s)] for each i in `starts`."""
    cnt = np.zeros(len(starts), np.int32)
    for k, p in enumerate(bytes(s)):
        col = M[p]
        if col.any():
            cnt += col[g[starts + k]]
    return cnt


def restate_finder(text, pattern):
    """finder_cpu (cas-offinder.cl:157-213) over every start of `text` (the
    reference's genome string), in work-item order: (loci, flags) with flag
    0 both strands, 1 forward only, 2 reverse only.  Windows holding ';' are
    dropped."""
    M = mismatch_table()
    g = np.frombuffer(bytes(text), np.uint8)
    L = len(pattern)
    npos = max(len(g) - L + 1, 0)
    starts = np.arange(npos, dtype=np.int64)
    fwd = _mismatch_counts(M, g, pattern, starts) > 0
    rev = _mismatch_counts(M, g, _revcomp_bytes(pattern), starts) > 0
    sep = np.convolve((g == ord(";")).astype(np.int32), np.ones(L, np.int32), "valid")[:npos] > 0
    flag = fwd.astype(np.int32) * 2 + rev.astype(np.int32)
    keep = (flag != 3) & ~sep
    return starts[keep], flag[keep]


def restate_comparer(text, loci, flags, comp, threshold):
    """comparer_cpu (cas-offinder.cl:214-286) for one compare string: hits as
    (start, '-' strand, mismatches), ordered by candidate then '+' before '-'.
    The reference stops counting past the threshold and then drops the
    candidate, so a full count gives the same hits."""
    M = mismatch_table()
    g = np.frombuffer(bytes(text), np.uint8)
    loci = np.asarray(loci, np.int64)
    flags = np.asarray(flags)
    fwd = _mismatch_counts(M, g, comp, loci)
    rev = _mismatch_counts(M, g, _revcomp_bytes(comp), loci)
    out = []
    for i, f, a, b in zip(loci.tolist(), flags.tolist(), fwd.tolist(), rev.tolist()):
        if f in (0, 1) and a <= threshold:
            out.append((i, False, a))
        if f in (0, 2) and b <= threshold:
            out.append((i, True, b))
    return out
