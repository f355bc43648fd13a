"""Python binding of libcasoff.so, the GB300 Cas-OFFinder search engine.

The engine itself is CUDA C++ behind the C ABI of include/cof.h; this module
only loads that library with ctypes.  `CasOFFinder` mirrors the reference's
engine class (Cas_OFFinder, cas-offinder.h:24-107): readInputFile,
setChrData*, search (loadNextChunk + findPattern + compareAll), and the
summary table.  Kernel-level calls with the OpenCL kernels' argument contracts
are `finder_chunk` / `comparer_chunk`.

There is no CPU fallback: importing works without a GPU, but opening an
engine raises if the library or a CUDA device is missing.

Because the directory name contains a hyphen, load this package with
`load_package()` from a checkout (or importlib) as `cas_offinder_gb300`.
"""
import ctypes
import os
import struct

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libcasoff.so")
CLI_PATH = os.path.join(PKG_DIR, "bin", "cas-offinder")

COF_OK = 0
STATUS_NAMES = {0: "OK", 1: "CUDA", 2: "ARG", 3: "NOMEM", 4: "INPUT", 5: "IO", 6: "STATE",
                7: "UNSUPPORTED", 8: "NOT_GENOME", 9: "DEVICE", 10: "TOO_LARGE", 11: "TIMEOUT"}
HEADER = ("##Generated by Cas-OFFinder 3.0.0\n"
          "#Id\tBulge Type\tcrRNA\tDNA\tChromosome\tLocation\tDirection\tMismatches\tBulge Size\n")

# Every entry point include/cof.h declares (checked by the CPU tests).
EXPORTS = [
    "cof_open", "cof_close", "cof_last_error", "cof_open_error", "cof_read_input", "cof_genome_path",
    "cof_input_info", "cof_genome_load_file", "cof_genome_load_text", "cof_genome_load_planes", "cof_search_planes", "cof_search_stream", "cof_set_autotune", "cof_schedule_text",
    "cof_genome_info", "cof_search", "cof_last_hit_count", "cof_set_summary", "cof_summary_text",
    "cof_header_text", "cof_finder_chunk", "cof_comparer_chunk", "cof_plane_words", "cof_pack_text",
    "cof_set_profiling", "cof_kernel_stats", "cof_reset_stats", "cof_timer_start", "cof_timer_stop",
    "cof_synchronize", "cof_set_comparer", "cof_comparer_info", "cof_search_chunk_static",
    "cof_batch_clear", "cof_batch_add_input", "cof_batch_size", "cof_job_rows", "cof_job_summary_text",
    "cof_server_start", "cof_server_submit", "cof_server_wait", "cof_server_release", "cof_server_stats",
    "cof_server_timing", "cof_server_set_step_segments",
    "cof_server_set_hit_reserve", "cof_server_memory", "cof_server_last_error", "cof_server_stop",
    "cof_router_open", "cof_router_add_genome", "cof_router_drop_genome", "cof_router_genomes", "cof_router_submit",
    "cof_router_wait", "cof_router_release", "cof_router_last_error", "cof_router_close",
    "cof_gzip_open", "cof_gzip_write", "cof_gzip_write_fn", "cof_gzip_close",
    "cofx_synth_record", "cofx_mismatch_table", "cofx_bs_programs", "cofx_genome_text",
]

# cof_write_fn: int (*)(void* ctx, const char* data, size_t len)
WRITE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t)

_lib = None


class CofError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"cof status {status} ({STATUS_NAMES.get(status, '?')}): {message}")
        self.status = status
        self.message = message


def build():
    """Compile libcasoff.so and the CLI in-tree (see build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_cof_build", os.path.join(PKG_DIR, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """The loaded libcasoff.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: build it with cas-offinder_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        c = ctypes
        vp, u64, u32, sz = c.c_void_p, c.c_uint64, c.c_uint32, c.c_size_t
        sig = {
            "cof_open": (c.c_int, [c.c_int, c.POINTER(vp)]),
            "cof_close": (None, [vp]),
            "cof_last_error": (c.c_char_p, [vp]),
            "cof_open_error": (c.c_char_p, []),
            "cof_read_input": (c.c_int, [vp, c.c_char_p, sz]),
            "cof_genome_path": (c.c_char_p, [vp]),
            "cof_input_info": (c.c_int, [vp, c.POINTER(u32), c.POINTER(u32), c.POINTER(u32)]),
            "cof_genome_load_file": (c.c_int, [vp, c.c_char_p]),
            "cof_genome_load_text": (c.c_int, [vp, c.c_char_p, u64, c.POINTER(c.c_char_p), c.POINTER(u64), u32]),
            "cof_genome_load_planes": (c.c_int, [vp, vp, vp, vp, u64, vp, vp, u64, c.POINTER(c.c_char_p),
                                                 c.POINTER(u64), u32]),
            "cof_search_planes": (c.c_int, [vp, vp, vp, vp, u64, vp, vp, u64, c.POINTER(c.c_char_p),
                                            c.POINTER(c.c_uint64), u32, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_genome_info": (c.c_int, [vp, c.POINTER(u64), c.POINTER(u32)]),
            "cof_search": (c.c_int, [vp, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_search_stream": (c.c_int, [vp, WRITE_FN, vp, c.POINTER(u64)]),
            "cof_set_autotune": (c.c_int, [vp, c.c_int]),
            "cof_schedule_text": (c.c_int, [vp, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_last_hit_count": (c.c_int, [vp, c.POINTER(u64), c.POINTER(u64)]),
            "cof_set_summary": (c.c_int, [vp, c.c_int]),
            "cof_summary_text": (c.c_int, [vp, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_header_text": (c.c_char_p, []),
            "cof_finder_chunk": (c.c_int, [vp, c.c_char_p, u64, c.c_char_p, u32, vp, vp, c.POINTER(u32)]),
            "cof_comparer_chunk": (c.c_int, [vp, c.c_char_p, u64, vp, vp, u32, c.c_char_p, u32, c.c_uint16,
                                             vp, vp, vp, c.POINTER(u32)]),
            "cof_plane_words": (u64, [u64]),
            "cof_pack_text": (u64, [vp, u64, vp, vp, vp, vp, vp]),
            "cof_set_profiling": (c.c_int, [vp, c.c_int]),
            "cof_kernel_stats": (c.c_int, [vp, c.c_char_p, c.POINTER(u64), c.POINTER(c.c_double),
                                           c.POINTER(c.c_double)]),
            "cof_reset_stats": (c.c_int, [vp]),
            "cof_synchronize": (c.c_int, [vp]),
            "cof_timer_start": (c.c_int, [vp]),
            "cof_set_comparer": (c.c_int, [vp, c.c_int]),
            "cof_comparer_info": (c.c_int, [vp, c.POINTER(c.c_int), c.POINTER(c.c_int)]),
            "cof_batch_clear": (c.c_int, [vp]),
            "cof_server_start": (c.c_int, [vp, u64, u64, u64, c.POINTER(vp)]),
            "cof_server_submit": (c.c_int, [vp, c.c_char_p, sz, c.POINTER(u64)]),
            "cof_server_wait": (c.c_int, [vp, u64, c.c_int, c.POINTER(c.c_void_p), c.POINTER(sz),
                                          c.POINTER(c.c_double)]),
            "cof_server_release": (c.c_int, [vp, u64]),
            "cof_server_timing": (c.c_int, [vp, u64] + [c.POINTER(c.c_double)] * 4),
            "cof_server_set_step_segments": (c.c_int, [vp, u32]),
            "cof_server_stats": (c.c_int, [vp] + [c.POINTER(u64)] * 6),
            "cof_server_set_hit_reserve": (c.c_int, [vp, u64]),
            "cof_server_memory": (c.c_int, [vp] + [c.POINTER(u64)] * 3),
            "cof_server_last_error": (c.c_char_p, [vp]),
            "cof_server_stop": (None, [vp]),
            "cof_router_open": (c.c_int, [c.c_int, u64, u64, u64, c.c_int, c.POINTER(vp)]),
            "cof_router_add_genome": (c.c_int, [vp, c.c_char_p, c.POINTER(u32)]),
            "cof_router_drop_genome": (c.c_int, [vp, c.c_char_p]),
            "cof_router_genomes": (c.c_int, [vp, c.POINTER(u32), c.POINTER(u32)]),
            "cof_router_submit": (c.c_int, [vp, c.c_char_p, sz, c.POINTER(u64)]),
            "cof_router_wait": (c.c_int, [vp, u64, c.c_int, c.POINTER(c.c_void_p), c.POINTER(sz),
                                          c.POINTER(c.c_double)]),
            "cof_router_release": (c.c_int, [vp, u64]),
            "cof_router_last_error": (c.c_char_p, [vp]),
            "cof_router_close": (None, [vp]),
            "cof_gzip_open": (c.c_int, [c.c_char_p, c.c_int, c.c_int, c.POINTER(vp)]),
            "cof_gzip_write": (c.c_int, [vp, c.c_char_p, sz]),
            "cof_gzip_write_fn": (c.c_int, [vp, c.c_char_p, sz]),
            "cof_gzip_close": (c.c_int, [vp]),
            "cof_batch_add_input": (c.c_int, [vp, c.c_char_p, sz, c.POINTER(u32)]),
            "cof_batch_size": (c.c_int, [vp, c.POINTER(u32)]),
            "cof_job_rows": (c.c_int, [vp, u32, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_job_summary_text": (c.c_int, [vp, u32, c.POINTER(c.c_void_p), c.POINTER(sz)]),
            "cof_search_chunk_static": (c.c_int, [vp, vp, vp, u64, c.c_char_p, c.c_char_p, u32, c.c_uint16, vp,
                                                  u64, vp, vp]),
            "cof_timer_stop": (c.c_int, [vp, c.POINTER(c.c_double)]),
            "cofx_mismatch_table": (None, [vp]),
            "cofx_bs_programs": (c.c_int, [c.c_char_p, sz, vp, vp, sz, vp, sz, vp, sz]),
            "cofx_genome_text": (c.c_int, [c.c_char_p, vp, u64, c.POINTER(u64)]),
            "cofx_synth_record": (u64, [u64, u32, u64, c.c_double, c.c_double, u32, c.c_double, u32, u32, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def _bytes_at(addr, n):
    """Copy n bytes at addr (ctypes.string_at takes a C int size: < 2 GiB only)."""
    return bytes((ctypes.c_char * n).from_address(addr)) if n else b""


# ---------------------------------------------------------------- packing
def mismatch_table():
    """The engine's mismatch predicate as a 256x256 uint8 array [pattern byte, genome byte]."""
    out = np.zeros(65536, np.uint8)
    lib().cofx_mismatch_table(_ptr(out))
    return out.reshape(256, 256)


def genome_text(path):
    """The reference's genome string for a FASTA / 2BIT file as the engine's
    loaders read it (host only), or None when the file is neither."""
    n = ctypes.c_uint64()
    p = os.fsencode(path)
    if lib().cofx_genome_text(p, None, 0, ctypes.byref(n)) != 0:
        return None
    out = ctypes.create_string_buffer(max(n.value, 1))
    lib().cofx_genome_text(p, out, n.value, ctypes.byref(n))
    return out.raw[:n.value]


def bs_programs(text):
    """The bit-sliced comparer's lane programs for one input file (test hook):
    dict with chunks, m, slots, row, prog / pgid (uint32 arrays), the
    variants as (key, threshold) in id order and `narrow` (the counts fit
    bit_width(slots) planes)."""
    import numpy as np
    raw = text.encode() if isinstance(text, str) else bytes(text)
    info = np.zeros(7, dtype=np.uint32)
    st = lib().cofx_bs_programs(raw, len(raw), _ptr(info), None, 0, None, 0, None, 0)
    if st != 0:
        raise CofError(st, "input does not fit the bit-sliced comparer" if st == 2 else "parse error")
    chunks, m, slots, row, nvar, kb, narrow = (int(x) for x in info)
    prog = np.zeros(max(chunks, 1) * (1 + slots // 2 + 2 * (m // 2)) * 32, dtype=np.uint32)
    pgid = np.zeros(max(chunks, 1) * m * 32, dtype=np.uint32)
    keys = ctypes.create_string_buffer(kb + 1)
    lib().cofx_bs_programs(raw, len(raw), _ptr(info), _ptr(prog), prog.size, _ptr(pgid), pgid.size, keys, kb + 1)
    variants = [(ln.split("\t")[0], int(ln.split("\t")[1])) for ln in keys.raw[:kb].decode().splitlines()]
    return {"chunks": chunks, "m": m, "slots": slots, "row": row, "prog": prog, "pgid": pgid, "variants": variants,
            "narrow": bool(narrow)}


def plane_words(n):
    return int(lib().cof_plane_words(n))


def _addr(seq):
    """Address of a bytes/bytearray buffer (bytes are copied once)."""
    if isinstance(seq, bytearray):
        return ctypes.addressof((ctypes.c_char * max(1, len(seq))).from_buffer(seq)) if len(seq) else None, seq
    keep = ctypes.create_string_buffer(bytes(seq), max(1, len(seq)))
    return ctypes.addressof(keep), keep


def pack_text(seq, out=None):
    """Pack a reference-style genome string into (hi, lo, ot, exc_pos, exc_byte)
    numpy arrays.  `out` = optional preallocated (hi, lo, ot) arrays."""
    L = lib()
    n = len(seq)
    W = plane_words(n)
    addr, keep = _addr(seq)
    if out is None:
        hi, lo, ot = np.zeros(W, np.uint32), np.zeros(W, np.uint32), np.zeros(W, np.uint32)
    else:
        hi, lo, ot = out
    ne = int(L.cof_pack_text(addr, n, _ptr(hi), _ptr(lo), _ptr(ot), None, None))
    ep = np.zeros(ne, np.uint64)
    eb = np.zeros(ne, np.uint8)
    if ne:
        L.cof_pack_text(addr, n, _ptr(hi), _ptr(lo), _ptr(ot), _ptr(ep), _ptr(eb))
    del keep
    return hi, lo, ot, ep, eb


# ---------------------------------------------------------------- engine
class CasOFFinder:
    """One CUDA device, one resident genome, one parsed input (see include/cof.h)."""

    def __init__(self, device=0):
        L = lib()
        h = ctypes.c_void_p()
        st = L.cof_open(device, ctypes.byref(h))
        if st != COF_OK:
            raise CofError(st, L.cof_open_error().decode())
        self._L = L
        self._h = h

    def close(self):
        if self._h:
            self._L.cof_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != COF_OK:
            raise CofError(st, self._L.cof_last_error(self._h).decode(errors="replace"))

    # Cas_OFFinder::readInputFile (cas-offinder.cpp:696-751)
    def readInputFile(self, text):
        if isinstance(text, str):
            text = text.encode()
        self._check(self._L.cof_read_input(self._h, text, len(text)))

    def read_input_path(self, path):
        with open(path, "rb") as f:
            self.readInputFile(f.read())

    @property
    def chrdir(self):
        return self._L.cof_genome_path(self._h).decode()

    def input_info(self):
        a, b, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self._L.cof_input_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"pattern_len": a.value, "variants": b.value, "bulge_records": c.value}

    # read_fasta / read_twobit + setChrData
    def load_genome_file(self, path):
        self._check(self._L.cof_genome_load_file(self._h, os.fsencode(path)))

    def load_genome_text(self, seq: bytes, names, starts):
        arr_n = (ctypes.c_char_p * max(1, len(names)))(*[n.encode() if isinstance(n, str) else n for n in names])
        arr_s = (ctypes.c_uint64 * max(1, len(starts)))(*starts)
        self._check(self._L.cof_genome_load_text(self._h, seq, len(seq), arr_n, arr_s, len(names)))

    def load_genome_planes(self, hi, lo, ot, n, exc_pos, exc_byte, names, starts):
        arr_n = (ctypes.c_char_p * max(1, len(names)))(*[x.encode() if isinstance(x, str) else x for x in names])
        arr_s = (ctypes.c_uint64 * max(1, len(starts)))(*starts)
        self._check(self._L.cof_genome_load_planes(
            self._h, _ptr(hi), _ptr(lo), _ptr(ot), n, _ptr(exc_pos), _ptr(exc_byte),
            0 if exc_pos is None else exc_pos.size, arr_n, arr_s, len(names)))

    def genome_info(self):
        n, r = ctypes.c_uint64(), ctypes.c_uint32()
        self._check(self._L.cof_genome_info(self._h, ctypes.byref(n), ctypes.byref(r)))
        return n.value, r.value

    # loadNextChunk + findPattern + compareAll
    def search(self) -> bytes:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_search(self._h, ctypes.byref(p), ctypes.byref(n)))
        return _bytes_at(p.value, n.value)

    def search_planes_view(self, hi, lo, ot, n, exc_pos, exc_byte, names, starts):
        """Load + search in one call (cof_search_planes): the plane upload
        overlaps the scan.  Returns (address, length) of the rows."""
        arr_n = (ctypes.c_char_p * max(1, len(names)))(*[x.encode() if isinstance(x, str) else x for x in names])
        arr_s = (ctypes.c_uint64 * max(1, len(starts)))(*starts)
        p, m = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_search_planes(
            self._h, _ptr(hi), _ptr(lo), _ptr(ot), n, _ptr(exc_pos), _ptr(exc_byte),
            0 if exc_pos is None else exc_pos.size, arr_n, arr_s, len(names), ctypes.byref(p), ctypes.byref(m)))
        return p.value, m.value

    def search_stream(self, write):
        """cof_search_stream: write(bytes) is called with the rows, chunk by
        chunk, in order; returns the total bytes written.  A write that
        raises stops the search (COF_ERR_IO)."""
        def cb(ctx, data, n):
            try:
                write(_bytes_at(data, n))
                return 0
            except Exception:
                return 1
        fn = WRITE_FN(cb)
        total = ctypes.c_uint64()
        self._check(self._L.cof_search_stream(self._h, fn, None, ctypes.byref(total)))
        return total.value

    def search_view(self):
        """(address, length) of the rows in the engine's pinned buffer, without a copy."""
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_search(self._h, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    # batched search (several input files over the resident genome)
    def batch_clear(self):
        self._check(self._L.cof_batch_clear(self._h))

    def batch_add_input(self, text):
        if isinstance(text, str):
            text = text.encode()
        j = ctypes.c_uint32()
        self._check(self._L.cof_batch_add_input(self._h, text, len(text), ctypes.byref(j)))
        return j.value

    def batch_size(self):
        n = ctypes.c_uint32()
        self._check(self._L.cof_batch_size(self._h, ctypes.byref(n)))
        return n.value

    def job_rows(self, job) -> bytes:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_job_rows(self._h, job, ctypes.byref(p), ctypes.byref(n)))
        return _bytes_at(p.value, n.value)

    def job_summary(self, job) -> bytes:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_job_summary_text(self._h, job, ctypes.byref(p), ctypes.byref(n)))
        return ctypes.string_at(p.value, n.value) if n.value else b""

    def last_hit_count(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.cof_last_hit_count(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_summary(self, on=True):
        self._check(self._L.cof_set_summary(self._h, 1 if on else 0))

    def summary(self) -> bytes:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_summary_text(self._h, ctypes.byref(p), ctypes.byref(n)))
        return ctypes.string_at(p.value, n.value) if n.value else b""

    # kernel-level entry points (OpenCL argument contracts)
    def finder_chunk(self, chr_bytes: bytes, worksize: int, pat2: bytes, patternlen: int):
        loci = np.zeros(max(1, worksize), np.uint32)
        flag = np.zeros(max(1, worksize), np.uint8)
        cnt = ctypes.c_uint32()
        self._check(self._L.cof_finder_chunk(self._h, chr_bytes, worksize, pat2, patternlen, _ptr(loci),
                                             _ptr(flag), ctypes.byref(cnt)))
        return loci[:cnt.value].copy(), flag[:cnt.value].copy()

    def comparer_chunk(self, chr_bytes: bytes, loci, flag, comp: bytes, threshold: int):
        loci = np.ascontiguousarray(loci, np.uint32)
        flag = np.ascontiguousarray(flag, np.uint8)
        cap = max(1, 2 * loci.size)
        mm_loci = np.zeros(cap, np.uint32)
        mm_count = np.zeros(cap, np.uint16)
        direction = np.zeros(cap, np.uint8)
        cnt = ctypes.c_uint32()
        self._check(self._L.cof_comparer_chunk(self._h, chr_bytes, len(chr_bytes), _ptr(loci), _ptr(flag),
                                               loci.size, comp, len(comp), threshold, _ptr(mm_loci),
                                               _ptr(mm_count), _ptr(direction), ctypes.byref(cnt)))
        k = cnt.value
        return mm_loci[:k].copy(), mm_count[:k].copy(), direction[:k].tobytes()

    def set_comparer(self, kind):
        """0 auto (bit-sliced when it fits), 1 popcount, 2 bit-sliced."""
        self._check(self._L.cof_set_comparer(self._h, kind))

    def set_autotune(self, on=True):
        self._check(self._L.cof_set_autotune(self._h, 1 if on else 0))

    def schedule(self):
        """Per pattern group: pattern, variants, slots, program length m,
        chunks and the autotuner's timings (one line each)."""
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self._L.cof_schedule_text(self._h, ctypes.byref(p), ctypes.byref(n)))
        return _bytes_at(p.value, n.value).decode()

    def comparer_info(self):
        k, sl = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.cof_comparer_info(self._h, ctypes.byref(k), ctypes.byref(sl)))
        return {"kind": {1: "popcount", 2: "bit-sliced"}[k.value], "slots": sl.value}

    # instrumentation
    def set_profiling(self, on=True):
        self._check(self._L.cof_set_profiling(self._h, 1 if on else 0))

    def reset_stats(self):
        self._check(self._L.cof_reset_stats(self._h))

    def kernel_stats(self, name):
        a, b, c = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cof_kernel_stats(self._h, name.encode(), ctypes.byref(a), ctypes.byref(b),
                                             ctypes.byref(c)))
        return {"launches": a.value, "ms": b.value, "units": c.value}

    def synchronize(self):
        self._check(self._L.cof_synchronize(self._h))

    def timer_start(self):
        self._check(self._L.cof_timer_start(self._h))

    def timer_stop(self):
        ms = ctypes.c_double()
        self._check(self._L.cof_timer_stop(self._h, ctypes.byref(ms)))
        return ms.value


class Server:
    """Served mode over an engine's resident genome (see include/cof.h).
    While it runs, use the engine only through this server."""

    def __init__(self, engine, max_active_variants=0, hit_buffer_bytes=0, segment_positions=0):
        self._L = engine._L
        self._eng = engine
        s = ctypes.c_void_p()
        st = self._L.cof_server_start(engine._h, max_active_variants, hit_buffer_bytes, segment_positions,
                                      ctypes.byref(s))
        if st != COF_OK:
            raise CofError(st, self._L.cof_last_error(engine._h).decode())
        self._s = s

    def submit(self, text):
        if isinstance(text, str):
            text = text.encode()
        t = ctypes.c_uint64()
        st = self._L.cof_server_submit(self._s, text, len(text), ctypes.byref(t))
        if st != COF_OK:
            raise CofError(st, self._L.cof_server_last_error(self._s).decode())
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        """(rows bytes, latency ms), or None on timeout."""
        p, n, lat = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_double()
        st = self._L.cof_server_wait(self._s, ticket, timeout_ms, ctypes.byref(p), ctypes.byref(n),
                                     ctypes.byref(lat))
        if st == 11:
            return None
        if st != COF_OK:
            raise CofError(st, self._L.cof_server_last_error(self._s).decode())
        rows = _bytes_at(p.value, n.value)
        self._L.cof_server_release(self._s, ticket)
        return rows, lat.value

    def wait_view(self, ticket, timeout_ms=-1):
        """(rows address, rows length, latency ms) without copying the rows,
        or None on timeout; the rows stay valid until release(ticket)."""
        p, n, lat = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_double()
        st = self._L.cof_server_wait(self._s, ticket, timeout_ms, ctypes.byref(p), ctypes.byref(n),
                                     ctypes.byref(lat))
        if st == 11:
            return None
        if st != COF_OK:
            raise CofError(st, self._L.cof_server_last_error(self._s).decode())
        return p.value, n.value, lat.value

    def release(self, ticket):
        self._L.cof_server_release(self._s, ticket)

    def timing(self, ticket):
        """Latency stages of a finished request (ms): admission, build, ring, format."""
        vals = [ctypes.c_double() for _ in range(4)]
        st = self._L.cof_server_timing(self._s, ticket, *[ctypes.byref(v) for v in vals])
        if st != COF_OK:
            raise CofError(st, "cof_server_timing")
        return dict(zip(("admission", "build", "ring", "format"), (v.value for v in vals)))

    def stats(self):
        vals = [ctypes.c_uint64() for _ in range(6)]
        self._L.cof_server_stats(self._s, *[ctypes.byref(v) for v in vals])
        keys = ("steps", "admitted", "completed", "pending", "active", "max_active")
        return dict(zip(keys, (v.value for v in vals)))

    def set_step_segments(self, k):
        """Ring segments one server step searches at most (default 4)."""
        st = self._L.cof_server_set_step_segments(self._s, int(k))
        if st != COF_OK:
            raise CofError(st, "cof_server_set_step_segments")

    def set_hit_reserve(self, nbytes):
        """Hit memory charged per running request at least, for admission."""
        self._L.cof_server_set_hit_reserve(self._s, int(nbytes))

    def memory(self):
        vals = [ctypes.c_uint64() for _ in range(3)]
        self._L.cof_server_memory(self._s, *[ctypes.byref(v) for v in vals])
        return dict(zip(("held_hit_bytes", "max_held_hit_bytes", "queue_bytes"), (v.value for v in vals)))

    def stop(self):
        if self._s:
            self._L.cof_server_stop(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()


class Router:
    """Served mode over several resident genomes (see include/cof.h): each
    request goes to the genome its input file's first line names."""

    def __init__(self, device=0, max_active_variants=0, hit_buffer_bytes=0, segment_positions=0, auto_load=False):
        self._L = lib()
        r = ctypes.c_void_p()
        st = self._L.cof_router_open(device, max_active_variants, hit_buffer_bytes, segment_positions,
                                     1 if auto_load else 0, ctypes.byref(r))
        if st != COF_OK:
            raise CofError(st, "cof_router_open failed")
        self._r = r

    def _err(self, st):
        return CofError(st, self._L.cof_router_last_error(self._r).decode())

    def add_genome(self, path):
        """Loads a genome file or directory; returns the number of genome files kept."""
        n = ctypes.c_uint32()
        st = self._L.cof_router_add_genome(self._r, os.fsencode(path), ctypes.byref(n))
        if st != COF_OK:
            raise self._err(st)
        return n.value

    def drop_genome(self, path):
        st = self._L.cof_router_drop_genome(self._r, os.fsencode(path))
        if st != COF_OK:
            raise self._err(st)

    def genomes(self):
        """(resident genomes, resident genome files)."""
        a, b = ctypes.c_uint32(), ctypes.c_uint32()
        self._L.cof_router_genomes(self._r, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def submit(self, text):
        if isinstance(text, str):
            text = text.encode()
        t = ctypes.c_uint64()
        st = self._L.cof_router_submit(self._r, text, len(text), ctypes.byref(t))
        if st != COF_OK:
            raise self._err(st)
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        """(rows bytes, latency ms), or None on timeout; releases the ticket."""
        p, n, lat = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_double()
        st = self._L.cof_router_wait(self._r, ticket, timeout_ms, ctypes.byref(p), ctypes.byref(n),
                                     ctypes.byref(lat))
        if st == 11:
            return None
        if st != COF_OK:
            raise self._err(st)
        rows = _bytes_at(p.value, n.value)
        self._L.cof_router_release(self._r, ticket)
        return rows, lat.value

    def close(self):
        if self._r:
            self._L.cof_router_close(self._r)
            self._r = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def gzip_write(path, parts, level=1, threads=0):
    """Writes the byte strings `parts` to `path` through cof_gzip_* (no GPU)."""
    L = lib()
    z = ctypes.c_void_p()
    st = L.cof_gzip_open(os.fsencode(path), level, threads, ctypes.byref(z))
    if st != COF_OK:
        raise CofError(st, "cof_gzip_open failed")
    for p in parts:
        st = L.cof_gzip_write(z, p, len(p))
        if st != COF_OK:
            L.cof_gzip_close(z)
            raise CofError(st, "cof_gzip_write failed")
    st = L.cof_gzip_close(z)
    if st != COF_OK:
        raise CofError(st, "cof_gzip_close failed")


RATES_LIB_PATH = os.path.join(PKG_DIR, "lib", "libcofrates.so")
SYNTH_PATH = os.path.join(PKG_DIR, "bin", "cof-synth")


def pipe_rates(device=0):
    """Measured integer-pipe throughput (lane-ops/s): {'lop3', 'popc', 'iadd'}.
    From libcofrates.so, the measurement library built beside the engine."""
    L = ctypes.CDLL(RATES_LIB_PATH)
    L.cofx_pipe_rates.restype = ctypes.c_int
    L.cofx_pipe_rates.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 3
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    if L.cofx_pipe_rates(device, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)) != 0:
        raise RuntimeError("cofx_pipe_rates failed")
    return {"lop3": a.value, "popc": b.value, "iadd": c.value}


def d2h_rates(device=0, nbytes=1 << 30):
    """Device -> pinned host copy rates (bytes/s) of `nbytes`: {'dma': one
    cudaMemcpyAsync, 'sm': a kernel storing into the mapped host buffer,
    'dma2': two half-size copies on two streams at once}.
    From libcofrates.so, the measurement library built beside the engine."""
    L = ctypes.CDLL(RATES_LIB_PATH)
    L.cofx_d2h_rates.restype = ctypes.c_int
    L.cofx_d2h_rates.argtypes = [ctypes.c_int, ctypes.c_size_t] + [ctypes.POINTER(ctypes.c_double)] * 3
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    if L.cofx_d2h_rates(device, nbytes, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)) != 0:
        raise RuntimeError("cofx_d2h_rates failed")
    return {"dma": a.value, "sm": b.value, "dma2": c.value}


# ---------------------------------------------------------------- synthetic genomes
def synth_record(seed, record, length, gc=0.41, gc_drift=0.0, drift_window=100000, n_frac=0.0,
                 n_run_min=100, n_run_max=10000) -> bytearray:
    """One synthetic record (see include/cof_tools.h)."""
    out = bytearray(length)
    if length:
        buf = (ctypes.c_char * length).from_buffer(out)
        lib().cofx_synth_record(seed, record, length, gc, gc_drift, drift_window, n_frac, n_run_min, n_run_max,
                                ctypes.cast(buf, ctypes.c_void_p))
    return out


def record_lengths(seed, count, total, lo=47_000_000, hi=249_000_000):
    """`count` lengths drawn log-uniform in [lo, hi], rescaled to sum to `total`."""
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    lens = np.floor(raw / raw.sum() * total).astype(np.int64)
    lens[-1] += total - lens.sum()
    return [int(x) for x in lens]


def write_fasta(path, names, seqs, width=60):
    with open(path, "wb") as f:
        for name, s in zip(names, seqs):
            f.write(b">" + (name.encode() if isinstance(name, str) else name) + b"\n")
            mv = memoryview(bytes(s))
            for i in range(0, len(mv), width):
                f.write(mv[i:i + width])
                f.write(b"\n")


_TWOBIT_CODE = np.full(256, 0, np.uint8)
for _b, _c in ((b"T", 0), (b"C", 1), (b"A", 2), (b"G", 3), (b"t", 0), (b"c", 1), (b"a", 2), (b"g", 3)):
    _TWOBIT_CODE[_b[0]] = _c


def write_twobit(path, names, seqs, mask_blocks=None):
    """Write a UCSC .2bit file (version 0, little-endian).  Bytes other than
    ACGT become N blocks.  `mask_blocks`: optional per-record list of
    (start, size) soft-mask blocks."""
    names = [n.encode() if isinstance(n, str) else n for n in names]
    header = struct.pack("<IIII", 0x1A412743, 0, len(names), 0)
    index_size = sum(1 + len(n) + 4 for n in names)
    recs = []
    for i, s in enumerate(seqs):
        a = np.frombuffer(bytes(s), np.uint8)
        isn = ~np.isin(a, np.frombuffer(b"ACGTacgt", np.uint8))
        starts, sizes = [], []
        if isn.any():
            d = np.diff(np.concatenate(([0], isn.astype(np.int8), [0])))
            st = np.flatnonzero(d == 1)
            en = np.flatnonzero(d == -1)
            starts, sizes = st.tolist(), (en - st).tolist()
        codes = _TWOBIT_CODE[a]
        pad = (-len(codes)) % 4
        codes = np.concatenate((codes, np.zeros(pad, np.uint8))).reshape(-1, 4)
        packed = (codes[:, 0] << 6 | codes[:, 1] << 4 | codes[:, 2] << 2 | codes[:, 3]).astype(np.uint8)
        mb = (mask_blocks[i] if mask_blocks else []) or []
        rec = struct.pack("<II", len(a), len(starts))
        rec += struct.pack(f"<{len(starts)}I", *starts) + struct.pack(f"<{len(sizes)}I", *sizes)
        rec += struct.pack("<I", len(mb))
        rec += struct.pack(f"<{len(mb)}I", *[m[0] for m in mb]) + struct.pack(f"<{len(mb)}I", *[m[1] for m in mb])
        rec += struct.pack("<I", 0) + packed.tobytes()
        recs.append(rec)
    with open(path, "wb") as f:
        f.write(header)
        off = 16 + index_size
        for n, r in zip(names, recs):
            f.write(bytes([len(n)]) + n + struct.pack("<I", off))
            off += len(r)
        for r in recs:
            f.write(r)


def reference_text(seqs):
    """The reference's in-memory genome for records `seqs`: upper-cased,
    joined by ';', with the start offset of each record (read_fasta.cpp:41-45)."""
    starts, parts, pos = [], [], 0
    for i, s in enumerate(seqs):
        if i:
            parts.append(b";")
            pos += 1
        starts.append(pos)
        b = bytes(s).upper()
        parts.append(b)
        pos += len(b)
    return b"".join(parts), starts
