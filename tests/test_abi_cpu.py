"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (no GPU needed: nothing here launches a kernel)."""
import os
import re

from conftest import ROOT


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(cofx?_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols(P, built):
    L = P.lib()
    declared = declared_functions()
    assert len(declared) >= 20
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    assert declared <= set(P.EXPORTS) | declared
    assert set(P.EXPORTS) <= declared


def test_header_text_matches_reference(P, built):
    assert P.lib().cof_header_text().decode() == P.HEADER


def test_cli_built(P, built):
    assert os.access(P.CLI_PATH, os.X_OK)


def test_pack_text_roundtrip(P, built):
    import numpy as np
    seq = b"ACGTN;RYacgt*" * 7 + b"GATTACA"
    hi, lo, ot, ep, eb = P.pack_text(seq)
    assert hi.size == P.plane_words(len(seq))
    dec = []
    for p in range(len(seq)):
        w, b = p >> 5, p & 31
        h, l, o = (int(hi[w]) >> b) & 1, (int(lo[w]) >> b) & 1, (int(ot[w]) >> b) & 1
        if not o:
            dec.append("TCAG"[h * 2 + l])
        elif not h:
            dec.append(";" if l else "N")
        else:
            i = int(np.searchsorted(ep, p))
            assert ep[i] == p
            dec.append(chr(eb[i]))
    assert "".join(dec).encode() == seq
    # positions past the end read as separators
    for p in range(len(seq), hi.size * 32):
        w, b = p >> 5, p & 31
        assert (int(ot[w]) >> b) & 1 and (int(lo[w]) >> b) & 1 and not (int(hi[w]) >> b) & 1


def test_synth_record_deterministic(P, built):
    a = P.synth_record(7, 3, 200000, gc=0.41, gc_drift=0.1, n_frac=0.05)
    b = P.synth_record(7, 3, 200000, gc=0.41, gc_drift=0.1, n_frac=0.05)
    assert a == b
    gc = (a.count(b"G") + a.count(b"C")) / (len(a) - a.count(b"N"))
    assert 0.30 < gc < 0.52
    assert 0.02 < a.count(b"N") / len(a) < 0.08
