"""GB300-native (sm_103a) implementation of GolayPair's candidate-generation ->
PSD-filter -> sorted-PSD-matching path.

The product is the C ABI in include/golaypair_gb300.h, implemented by
golaypair_gb300/_build/libgolaypair_gb300.so (CUDA kernels + host runtime),
and the `golay` command line driver next to it, which mirrors the
reference's `main`.  This module is a thin ctypes binding used by tests and
benchmarks.  There is no CPU fallback: every call fails loudly when the
library is missing or no GB300 is present.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libgolaypair_gb300.so")
CLI_PATH = os.path.join(PKG, "_build", "golay")
HEADER = os.path.join(os.path.dirname(PKG), "include", "golaypair_gb300.h")

GP_PSD_FP64 = 0
GP_PSD_TC_GUARDED = 1
GP_FORMAT_TEXT = 0
GP_FORMAT_BINARY = 1

_lib = None


class GPError(RuntimeError):
    pass


class PsdStats(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("n_pass", ctypes.c_int64), ("n_unsure", ctypes.c_int64),
                ("guard", ctypes.c_float), ("err_coef", ctypes.c_float)]


class GenStats(ctypes.Structure):
    _fields_ = [("necklaces", ctypes.c_int64), ("candidates", ctypes.c_int64), ("psd_pass", ctypes.c_int64),
                ("written_a", ctypes.c_int64), ("written_b", ctypes.c_int64), ("unsure", ctypes.c_int64),
                ("seconds", ctypes.c_double)]


class GenJob(ctypes.Structure):
    """One job of gp_generate_batch: a word-rank window of one order."""
    _fields_ = [("order", ctypes.c_int), ("compress", ctypes.c_int), ("paf", ctypes.c_int),
                ("begin_hi", ctypes.c_uint64), ("begin_lo", ctypes.c_uint64), ("end_hi", ctypes.c_uint64),
                ("end_lo", ctypes.c_uint64), ("path_a", ctypes.c_char_p), ("path_b", ctypes.c_char_p)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("enum_variant", ctypes.c_int), ("windows_per_thread", ctypes.c_int), ("cand_cap", ctypes.c_int64),
                ("tc_ctas_per_sm", ctypes.c_int), ("no_graph", ctypes.c_int), ("iterations", ctypes.c_int),
                ("tune_seconds", ctypes.c_double), ("multi_launch", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build():
    from . import native_build
    return native_build.build()


def lib():
    """Loads the in-tree native library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GPError(f"native library missing: {LIB_PATH} (run golaypair_gb300.build())")
    L = ctypes.CDLL(LIB_PATH)
    P, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    cp = ctypes.c_char_p
    L.gp_ctx_create.argtypes = [ctypes.POINTER(P), i32]
    L.gp_ctx_destroy.argtypes = [P]
    L.gp_last_error.argtypes = [P]
    L.gp_last_error.restype = cp
    L.gp_device_sm_count.argtypes = [P]
    L.gp_psd_filter.argtypes = [P, P, i64, i32, i32, i32, i32, P, P]
    L.gp_psd_filter_device.argtypes = [P, P, i64, i32, i32, i32, i32, P, P, P]
    L.gp_psd_tc_values.argtypes = [P, P, i64, i32, P]
    L.gp_kernel_timing.argtypes = [P, i32]
    L.gp_kernel_time.argtypes = [P, P, P]
    L.gp_debug_tc_trace.argtypes = [P, i32, P, i32]
    L.gp_psd_fp64_values.argtypes = [P, P, i64, i32, P]
    for name, args in _STAGE_SIGS.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.argtypes = args
    L.gp_debug_pair_generator_count.restype = ctypes.c_int64
    L.gp_job_ranges.restype = ctypes.c_int64
    _lib = L
    return L


_P, _i32, _i64, _u64, _cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_char_p
_STAGE_SIGS = {
    "gp_generate": [_P, _i32, _i32, _i32, _i32, _i32, _cp, _cp, _P],
    "gp_generate_window": [_P, _i32, _i32, _i32, _u64, _u64, _u64, _u64, _cp, _cp, _P],
    "gp_generate_batch": [_P, _P, _i32, _i32, _P, _P],
    "gp_generate_resumable": [_P, _i32, _i32, _i32, _i32, _i32, _cp, _cp, _cp, _i32, ctypes.c_double, _P, _P],
    "gp_generate_window_resumable": [_P, _i32, _i32, _i32, _u64, _u64, _u64, _u64, _cp, _cp, _cp, _i32,
                                     ctypes.c_double, _P, _P],
    "gp_tuned_settings": [_P, _P, _i32],
    "gp_sort": [_P, _P, _i32, _cp],
    "gp_match": [_P, _i32, _i32, _i32, _cp, _cp, _cp, _i32, _P],
    "gp_uncompress": [_P, _i32, _i32, _i32, _i32, _cp, _cp, _cp, _cp],
    "gp_uncompress_lines": [_P, _i32, _i32, _i32, _i32, _cp, _cp, _cp, _cp, _i64, _i64, _i64],
    "gp_uncompress_chain": [_P, _i32, _P, _i32, _i32, _cp, _P, _i64, _i64, _i64],
    "gp_equiv_filter": [_P, _i32, _i32, _cp, _cp],
    "gp_set_output_format": [_P, _i32],
    "gp_export_text": [_P, _cp, _cp],
    "gp_set_spectral_prune": [_P, _i32],
    "gp_job_ranges": [_i32, _i32, _i32, _i32, _i32, _P, _i64],
    "gp_debug_wait_timeout": [_P, _i64],
    "gp_check": [_P, _P],
    "gp_debug_pair_generator_count": [_i32, _i32],
    "gp_debug_pair_group_check": [_i32, _i32],
}


def header_symbols():
    """Names of the functions include/golaypair_gb300.h declares."""
    import re
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(gp_\w+)\s*\(", text, re.M)))


def job_ranges(order, compress, paf, proc_id, proc_num):
    """gp_job_ranges: the word-rank ranges [begin, end) of job proc_id of
    proc_num (host only)."""
    L = lib()
    n = L.gp_job_ranges(order, compress, paf, proc_id, proc_num, None, 0)
    if n < 0:
        raise GPError(f"gp_job_ranges failed ({n})")
    buf = (ctypes.c_uint64 * (4 * max(n, 1)))()
    L.gp_job_ranges(order, compress, paf, proc_id, proc_num, buf, n)
    return [((buf[4 * i] << 64) | buf[4 * i + 1], (buf[4 * i + 2] << 64) | buf[4 * i + 3]) for i in range(n)]


def export_text(in_path, out_path):
    """gp_export_text without a context (host only): the text lines of a
    binary survivor file."""
    rc = lib().gp_export_text(None, str(in_path).encode(), str(out_path).encode())
    if rc != 0:
        raise GPError(f"gp_export_text failed ({rc}) on {in_path}")


class Context:
    """One gp_ctx on one GPU."""

    def __init__(self, device=0):
        self._lib = lib()
        self._h = ctypes.c_void_p()
        rc = self._lib.gp_ctx_create(ctypes.byref(self._h), device)
        if rc != 0:
            raise GPError(f"gp_ctx_create failed ({rc}): CUDA device {device} is not an sm_103a GPU or unusable")

    def close(self):
        if self._h:
            self._lib.gp_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def check(self, rc, what):
        if rc != 0:
            msg = self._lib.gp_last_error(self._h)
            raise GPError(f"{what} -> {rc}: {msg.decode() if msg else ''}")
        return rc

    @property
    def sm_count(self):
        return self._lib.gp_device_sm_count(self._h)

    def psd_filter(self, seqs, order, paf=0, mode=GP_PSD_TC_GUARDED):
        """Host-buffer batched PSD filter; returns (bool verdicts, PsdStats)."""
        seqs = np.ascontiguousarray(seqs, dtype=np.int8)
        n, L = seqs.shape
        mask = np.zeros((n + 31) // 32, dtype=np.uint32)
        st = PsdStats()
        self.check(self._lib.gp_psd_filter(self._h, seqs.ctypes.data, n, L, order, paf, mode, mask.ctypes.data,
                                           ctypes.byref(st)), "gp_psd_filter")
        return unpack_mask(mask, n), st

    def psd_filter_device(self, d_seqs_ptr, n, L, order, paf, mode, d_mask_ptr, stream_ptr=None, stats=False):
        """Device-buffer filter (pointers as ints); enqueued on stream_ptr."""
        st = PsdStats() if stats else None
        self.check(self._lib.gp_psd_filter_device(self._h, d_seqs_ptr, n, L, order, paf, mode, d_mask_ptr,
                                                  stream_ptr, ctypes.byref(st) if st is not None else None),
                   "gp_psd_filter_device")
        return st

    def check_stream(self, stream_ptr=None):
        """gp_check: waits for the stream and raises on a device-side error
        recorded by the context's kernels (timeout, overflow)."""
        self.check(self._lib.gp_check(self._h, stream_ptr), "gp_check")

    def psd_filter_host_raw(self, seqs_ptr, n, L, order, paf, mode, mask_ptr):
        """Host-buffer filter on raw pointers (e.g. pinned memory)."""
        st = PsdStats()
        self.check(self._lib.gp_psd_filter(self._h, seqs_ptr, n, L, order, paf, mode, mask_ptr, ctypes.byref(st)),
                   "gp_psd_filter")
        return st

    def set_spectral_prune(self, on):
        """Drop generation candidates that cannot have a complementary partner
        (gp_set_spectral_prune)."""
        self.check(self._lib.gp_set_spectral_prune(self._h, 1 if on else 0), "gp_set_spectral_prune")

    def set_output_format(self, fmt):
        """GP_FORMAT_TEXT or GP_FORMAT_BINARY for the generation files."""
        self.check(self._lib.gp_set_output_format(self._h, fmt), "gp_set_output_format")

    def generate_window(self, order, compress, paf, begin, end, path_a, path_b):
        """gp_generate_window over word ranks [begin, end); returns GenStats."""
        st = GenStats()
        m = (1 << 64) - 1
        self.check(self._lib.gp_generate_window(self._h, order, compress, paf, begin >> 64, begin & m, end >> 64,
                                                end & m, str(path_a).encode(), str(path_b).encode(),
                                                ctypes.byref(st)), "gp_generate_window")
        return st

    def generate_window_resumable(self, order, compress, paf, begin, end, path_a, path_b, checkpoint,
                                  max_iterations=0, max_seconds=0.0):
        """gp_generate_window_resumable; returns (done, GenStats)."""
        st = GenStats()
        done = ctypes.c_int(0)
        m = (1 << 64) - 1
        self.check(self._lib.gp_generate_window_resumable(
            self._h, order, compress, paf, begin >> 64, begin & m, end >> 64, end & m, str(path_a).encode(),
            str(path_b).encode(), str(checkpoint).encode(), max_iterations, float(max_seconds), ctypes.byref(done),
            ctypes.byref(st)), "gp_generate_window_resumable")
        return bool(done.value), st

    def generate_batch(self, jobs, autotune=False, config=None):
        """gp_generate_batch.  jobs: (order, compress, paf, begin, end,
        path_a, path_b) tuples.  Returns ([GenStats per job], BatchConfig)."""
        n = len(jobs)
        arr = (GenJob * n)()
        keep = []
        m = (1 << 64) - 1
        for i, (order, comp, paf, lo, hi, pa, pb) in enumerate(jobs):
            a, b = str(pa).encode(), str(pb).encode()
            keep += [a, b]
            arr[i] = GenJob(order, comp, paf, lo >> 64, lo & m, hi >> 64, hi & m, a, b)
        cfg = config if config is not None else BatchConfig()
        stats = (GenStats * n)()
        self.check(self._lib.gp_generate_batch(self._h, ctypes.cast(arr, ctypes.c_void_p), n, 1 if autotune else 0,
                                               ctypes.byref(cfg), ctypes.cast(stats, ctypes.c_void_p)),
                   "gp_generate_batch")
        return list(stats), cfg

    def tuned_settings(self):
        """{workload key: [values]} chosen by the context's tuners."""
        need = self._lib.gp_tuned_settings(self._h, None, 0)
        buf = ctypes.create_string_buffer(max(need, 1))
        self._lib.gp_tuned_settings(self._h, buf, len(buf))
        out = {}
        for line in buf.value.decode().splitlines():
            k, *v = line.split()
            out[k] = [int(x) for x in v]
        return out

    def kernel_timing(self, enable=True):
        self._lib.gp_kernel_timing(self._h, 1 if enable else 0)

    def kernel_time(self):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._lib.gp_kernel_time(self._h, ctypes.byref(ms), ctypes.byref(n))
        return ms.value, n.value

    TRACE_NAMES = ["conv_wait_raw", "conv_wait_a", "conv_work", "epi_wait_acc", "epi_ld", "epi_work",
                   "mma_wait_a", "mma_wait_acc", "mma_issue", "prod_wait", "prod_issue", "tiles", "conv_fence",
                   "mma_commit", "conv_st", "epi_tail"]

    def tc_trace(self, enable):
        """Reads (and resets) the tensor-core filter's per-role cycle counters."""
        out = (ctypes.c_uint64 * len(self.TRACE_NAMES))()
        self.check(self._lib.gp_debug_tc_trace(self._h, 1 if enable else 0, out, len(out)), "gp_debug_tc_trace")
        return dict(zip(self.TRACE_NAMES, list(out)))

    def psd_tc_values(self, seqs):
        seqs = np.ascontiguousarray(seqs, dtype=np.int8)
        n, L = seqs.shape
        out = np.zeros((n, L // 2), dtype=np.float32)
        self.check(self._lib.gp_psd_tc_values(self._h, seqs.ctypes.data, n, L, out.ctypes.data), "gp_psd_tc_values")
        return out

    def psd_fp64_values(self, seqs):
        seqs = np.ascontiguousarray(seqs, dtype=np.int8)
        n, L = seqs.shape
        out = np.zeros((n, L), dtype=np.float64)
        self.check(self._lib.gp_psd_fp64_values(self._h, seqs.ctypes.data, n, L, out.ctypes.data),
                   "gp_psd_fp64_values")
        return out


def unpack_mask(mask, n):
    bits = np.unpackbits(mask.view(np.uint8), bitorder="little")
    return bits[:n].astype(bool)
