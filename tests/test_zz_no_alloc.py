"""The allocation-free entry point cof_search_chunk_static against the
existing kernel-level entry points, through the C ABI.

Callers of cof_search_chunk_static cannot allocate device memory when they
search (their memory is reserved up front in their own pool, or they cannot
afford cudaMalloc's device-wide synchronization), so this test allocates the
genome planes and the hit buffer itself, as such a caller would, and checks
that two calls in a row -- which share the library's fixed scratch array --
each give exactly the hits of cof_finder_chunk + cof_comparer_chunk and of the
numpy restatement of finder_cpu/comparer_cpu (cases.py), with concrete, IUPAC,
lower-case and two-word (48-position) queries.  This file is collected last
so a failure here comes after every other test has run."""
import ctypes
import os

import numpy as np
import pytest

import cases
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

PATTERN = b"N" * 21 + b"GG"
RC = bytes.maketrans(b"ACGTRYKMHDBV", b"TGCAYRMKDHVB")


def chunk_text(P):
    seqs, cur = [], None
    for line in open(os.path.join(GOLDEN, "ngg_fasta", "genome.fa"), "rb").read().split(b"\n"):
        line = line.rstrip(b"\r")
        if line.startswith(b">"):
            cur = bytearray()
            seqs.append(cur)
        elif line:
            cur += line
    text, _ = P.reference_text(seqs)
    return text  # ~100 kbp with planted guide sites, two records


def expected_hits(P, eng, text, pattern, comp, thr):
    """(hits of cof_finder_chunk + cof_comparer_chunk, hits of the restatement)."""
    L = len(pattern)
    loci, flag = eng.finder_chunk(text, len(text) - L + 1, pattern + pattern[::-1].translate(RC), L)
    mm_loci, mm_count, direction = eng.comparer_chunk(text, loci, flag, comp, thr)
    chunk = sorted(zip(mm_loci.tolist(), [d == ord("-") for d in direction], mm_count.tolist()))
    rl, rf = cases.restate_finder(text, pattern.upper())
    return chunk, sorted(cases.restate_comparer(text, rl, rf, comp.upper(), thr))


def static_hits(P, torch, planes, n, pattern, comp, thr, cap=1 << 16):
    d_hits = torch.zeros(cap, dtype=torch.int64, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    st = P.lib().cof_search_chunk_static(
        ctypes.c_void_p(planes[0].data_ptr()), ctypes.c_void_p(planes[1].data_ptr()),
        ctypes.c_void_p(planes[2].data_ptr()), n, pattern, comp, len(pattern), thr,
        ctypes.c_void_p(d_hits.data_ptr()), cap, ctypes.c_void_p(d_count.data_ptr()),
        ctypes.c_void_p(stream.cuda_stream))
    assert st == P.COF_OK
    torch.cuda.synchronize()
    k = int(d_count.item())
    assert k <= cap
    keys = d_hits[:k].cpu().numpy().view(np.uint64)
    return sorted((int((x >> 8) & ((1 << 36) - 1)), bool((x >> 7) & 1), int(x & 0x7F)) for x in keys)


def test_static_chunk_search_matches_existing_entry_points(P, built):
    torch = pytest.importorskip("torch")
    text = chunk_text(P)
    n = len(text)
    hi, lo, ot, _, _ = P.pack_text(text)
    planes = [torch.from_numpy(a.view(np.int32)).cuda() for a in (hi, lo, ot)]
    queries = [(PATTERN, b"GGCCGACCTGTCGCTGACGCNNN", 9), (PATTERN, b"ACGTRYACGTACGTACGTACNNN", 9),
               (PATTERN.lower(), b"ggccrACCTGYCGCTGAsgcNNN", 8),
               (b"N" * 45 + b"NGG", b"GGCCGACCTGTCGCTGACGCAGTCRYACGGTTACGATCGATCGAANNN", 26)]
    with P.CasOFFinder(0) as eng:
        want = []
        for pat, c, t in queries:
            chunk, restated = expected_hits(P, eng, text, pat.upper(), c.upper(), t)
            assert chunk == restated, c
            assert len(chunk) > 0, c
            want.append(chunk)
    for (pat, comp, thr), exp in zip(queries, want):  # calls in a row share the scratch array
        assert static_hits(P, torch, planes, n, pat, comp, thr) == exp, comp
    # A chunk above the fixed limit is rejected without touching the device.
    big = (1 << 21) + 1
    st = P.lib().cof_search_chunk_static(
        ctypes.c_void_p(planes[0].data_ptr()), ctypes.c_void_p(planes[1].data_ptr()),
        ctypes.c_void_p(planes[2].data_ptr()), big, PATTERN, queries[0][0], len(PATTERN), 4,
        ctypes.c_void_p(planes[0].data_ptr()), 1, ctypes.c_void_p(planes[0].data_ptr()), None)
    assert st == 10  # COF_ERR_TOO_LARGE
