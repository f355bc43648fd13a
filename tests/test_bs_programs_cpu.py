"""Lane programs of the bit-sliced comparer (host logic, no GPU).

A lane program counts its first variant in full and reaches each later one by
steps that add one class word and remove one.  Replaying the programs as set
operations must produce every compare variant exactly once, with exactly its
own slots and its own threshold bias -- whatever chains the builder chose."""
import random

import pytest

CLASS = {c: i + 1 for i, c in enumerate("TCAGVDBHRYKMWS")}  # row of a pattern byte; others never mismatch


def bit_width(s):
    b = 1
    while (1 << b) <= s:
        b += 1
    return b


def replay(P, text):
    r = P.bs_programs(text)
    S, m, row = r["slots"], r["m"], r["row"]
    words = 1 + S // 2 + 2 * (m // 2)
    prog = r["prog"].reshape(max(r["chunks"], 1), words * 32)
    pgid = r["pgid"].reshape(max(r["chunks"], 1), m, 32)
    nb = bit_width(S)
    seen = {}
    for c in range(r["chunks"]):
        for lane in range(32):
            hdr = int(prog[c, lane])
            cur = set()
            for w in range(S // 2):
                pk = int(prog[c, (1 + w) * 32 + lane])
                for off in (pk & 0xFFFF, pk >> 16):
                    if off:
                        assert off not in cur
                        cur.add(off)
            kadd = hdr & 0xFF
            out = []
            if hdr & 0x100:
                out.append((int(pgid[c, 0, lane]), frozenset(cur), kadd))
            else:
                assert not cur
            for st in range(2 * (m // 2)):
                w = int(prog[c, (1 + S // 2) * 32 + ((st // 2) * 32 + lane) * 2 + st % 2])
                if st >= m - 1:
                    assert w == 0, "padding step"
                add, rem, emit = w & 0x7FFF, w >> 16, bool(w & 0x8000)
                assert rem < 0x8000
                if rem:
                    assert rem in cur, "a step removes a word the count does not hold"
                    cur.remove(rem)
                if add:
                    assert add not in cur
                    cur.add(add)
                # the biased counter never overflows its NB + 1 planes
                assert len(cur) <= S + 1
                if emit:
                    out.append((int(pgid[c, st + 1, lane]), frozenset(cur), kadd))
            for gid, slots, k in out:
                assert gid not in seen, f"variant {gid} tested twice"
                seen[gid] = (slots, k)
    variants = r["variants"]
    assert sorted(seen) == list(range(len(variants))), "every variant exactly once"
    for gid, (key, thr) in enumerate(variants):
        want = frozenset((CLASS[ch] * row + (k + CLASS[ch]) % row) * 8 for k, ch in enumerate(key) if ch in CLASS)
        slots, k = seen[gid]
        assert slots == want, f"variant {gid} ({key}) counted over the wrong slots"
        assert len(want) <= S
        assert k == (1 << nb) - 1 - min(thr, (1 << nb) - 1)
    return r


def guide_input(guides, pattern, dna, rna, genome="g.fa"):
    head = pattern + (f" {dna} {rna}" if dna or rna else "")
    return "\n".join([genome, head] + [f"{g} {mm}" for g, mm in guides]) + "\n"


def rand_guide(rng, n, alphabet="ACGT"):
    return "".join(rng.choice(alphabet) for _ in range(n))


def test_plain_workload_chains(P):
    """NRG, DNA bulge 2, RNA bulge 1, four 20-nt guides: bulge variants chain,
    so far fewer than one lane per variant is needed."""
    rng = random.Random(3)
    guides = [(rand_guide(rng, 20) + "NNN", 5) for _ in range(4)]
    r = replay(P, guide_input(guides, "N" * 21 + "RG", 2, 1))
    assert len(r["variants"]) > 200
    assert r["m"] > 1
    assert r["chunks"] * 32 < len(r["variants"])


@pytest.mark.parametrize("seed", range(6))
def test_random_inputs(P, seed):
    rng = random.Random(100 + seed)
    pam5 = seed % 2 == 1
    pam = rng.choice(["NGG", "NRG", "NNGRRT", "TTTV", "NAG"])
    spacer = rng.randint(12, 24)
    dna, rna = rng.randint(0, 2), rng.randint(0, 2)
    if pam5:
        pam = rng.choice(["TTTV", "TTTN"])
        pattern = pam + "N" * spacer
    else:
        pattern = "N" * spacer + pam
    guides = []
    for i in range(rng.randint(1, 12)):
        g = rand_guide(rng, spacer, "ACGT" if i % 3 else "ACGTRYKMSWN")
        guides.append(((("N" * len(pam)) + g) if pam5 else (g + "N" * len(pam)), rng.randint(0, 8)))
    # a duplicate guide with another threshold (first inserter wins) and an
    # all-threshold guide
    guides.append((guides[0][0], 1))
    guides.append((guides[-2][0], 65535 % 65536))
    replay(P, guide_input(guides, pattern, dna, rna))


def test_homopolymer_and_wide_thresholds(P):
    guides = [("A" * 20 + "NGG", 3), ("ACGTACGTAAAACCCCGGGG" + "NGG", 0), ("T" * 20 + "NGG", 40)]
    replay(P, guide_input(guides, "N" * 20 + "NGG", 2, 2))


def test_single_variant(P):
    r = replay(P, guide_input([("ACGTACGTACGTACGTACGT" + "NGG", 4)], "N" * 20 + "NGG", 0, 0))
    assert r["chunks"] == 1 and r["m"] == 1


# ---------------------------------------------------------------- counters

def programs_of(r):
    """The lane programs as (kadd, first slots or None, first id, steps), a
    step being (added, removed, testing, id)."""
    S, m = r["slots"], r["m"]
    words = 1 + S // 2 + 2 * (m // 2)
    prog = r["prog"].reshape(max(r["chunks"], 1), words * 32)
    pgid = r["pgid"].reshape(max(r["chunks"], 1), m, 32)
    out = []
    for c in range(r["chunks"]):
        for lane in range(32):
            hdr = int(prog[c, lane])
            first = set()
            for w in range(S // 2):
                pk = int(prog[c, (1 + w) * 32 + lane])
                first.update(off for off in (pk & 0xFFFF, pk >> 16) if off)
            steps = []
            for st in range(m - 1):
                w = int(prog[c, (1 + S // 2) * 32 + ((st // 2) * 32 + lane) * 2 + st % 2])
                steps.append((w & 0x7FFF, w >> 16, bool(w & 0x8000), int(pgid[c, st + 1, lane])))
            out.append((hdr & 0xFF, first if hdr & 0x100 else None, int(pgid[c, 0, lane]), steps))
    return out


def counter_errors(r, narrow, rng, candidates=300):
    """Runs every lane program over random candidates with the kernel's
    counter arithmetic -- count + bias held modulo 2^NP (NP = NB count planes
    when narrow and the programs have steps, else NB + 1), each step adding
    its added word's mismatch and subtracting its removed word's, a test
    passing where the top plane is clear and reporting planes - bias -- and
    returns how many tests disagree with counting the variant's slots
    directly."""
    S, m = r["slots"], r["m"]
    nb = bit_width(S)
    np_ = nb if (narrow and m > 1) else nb + 1
    mod, half = 1 << np_, 1 << (nb - 1)
    progs = programs_of(r)
    thr = [t for _, t in r["variants"]]
    offs = sorted({o for _, f, _, st in progs for o in (f or ())} | {x for *_, st in progs for a, b, _, _ in st
                                                                      for x in (a, b) if x})
    errors = 0
    for _ in range(candidates):
        # from near-misses to all positions mismatching (the largest sums)
        p = rng.choice([0.02, 0.1, 0.3, 0.75, 0.95, 1.0])
        mm = {o: int(rng.random() < p) for o in offs}
        for kadd, first, gid0, steps in progs:
            bias = kadd - half if np_ == nb else kadd
            cur = set(first or ())
            ctr = (sum(mm[o] for o in cur) + bias) % mod
            tests = [(gid0, frozenset(cur), ctr)] if first is not None else []
            for add, rem, testing, gid in steps:
                if rem:
                    cur.remove(rem)
                if add:
                    cur.add(add)
                ctr = (ctr + (mm[add] if add else 0) - (mm[rem] if rem else 0)) % mod
                if testing:
                    tests.append((gid, frozenset(cur), ctr))
            for gid, slots, c in tests:
                direct = sum(mm[o] for o in slots)
                passes = not (c >> (np_ - 1)) & 1
                if passes != (direct <= thr[gid]) or (passes and c - bias != direct):
                    errors += 1
    return errors


@pytest.mark.parametrize("case", ["plain", "edges_narrow", "edges_wide", "random"])
def test_counter_planes(P, case):
    """The narrow counters (bit_width(slots) planes) decide and decode every
    test exactly where the library allows them, and so do NB + 1 planes
    everywhere."""
    rng = random.Random("counters-" + case)
    if case == "plain":
        guides = [(rand_guide(rng, 20) + "NNN", 5) for _ in range(4)]
        text, want = guide_input(guides, "N" * 21 + "RG", 2, 1), True
    elif case == "edges_narrow":  # 20 positions: thresholds 4 and 15 fit 5 planes
        guides = [(rand_guide(rng, 20) + "NNN", t) for t in (4, 15, 4)]
        text, want = guide_input(guides, "N" * 21 + "RG", 1, 1), True
    elif case == "edges_wide":  # 3 needs a sixth plane (20 - 3 > 16), so does 16
        guides = [(rand_guide(rng, 20) + "NNN", t) for t in (3, 16, 5)]
        text, want = guide_input(guides, "N" * 21 + "RG", 1, 1), False
    else:
        guides = [(rand_guide(rng, 21, "ACGTRYKMSWN") + "NN", rng.randint(0, 8)) for _ in range(6)]
        text, want = guide_input(guides, "N" * 21 + "RG", 2, 1), None
    r = P.bs_programs(text)
    if want is not None:
        assert r["narrow"] == want
    assert counter_errors(r, r["narrow"], rng) == 0
    assert counter_errors(r, False, rng) == 0
    if not r["narrow"] and r["m"] > 1 and case == "edges_wide":
        # the condition is needed: forcing NB planes here misjudges tests
        # (a 20-mismatch window wraps to a clear top plane under threshold 3)
        assert counter_errors(r, True, rng) > 0
