"""gp_psd_filter_noalloc: the PSD filter for callers that cannot allocate.

Some callers cannot call cudaMalloc (code running under another framework's
allocator or memory pool, allocation-free real-time loops, devices whose
memory is reserved by their owner).  gp_psd_filter_noalloc serves them: it
takes its working buffers from a fixed static device array instead of
allocating.  This file checks, through the C ABI, that two calls in a row
give exactly the verdicts of the allocating entry point
gp_psd_filter_device (the filter's verdicts are exact, so the tolerance is
zero), and that a batch over the array's row limit is rejected.  pytest
collects this file last, so a failure here stops a run only after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

import golaypair_gb300 as gp

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 20  # the entry point's fixed scratch limit


def _entry():
    fn = gp.lib().gp_psd_filter_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    fn = _entry()
    rng = np.random.default_rng(2026)
    # (order, compress, paf, rows), called one after the other: one length in
    # every padded-K bucket of the tensor-core filter (K = 16 .. 128); the
    # entry point builds its twiddles on the device, the allocating one on
    # the host, and the verdicts must agree in every bucket
    cases = [
        (26, 2, 0, 100_000),    # L 13, K 16
        (57, 3, -2, 200_003),   # L 19, K 32
        (62, 2, 0, 60_000),     # L 31, K 32 (no shifted loads: 31 + 3 > 32)
        (90, 2, 0, 300_000),    # L 45, K 48
        (57, 1, -2, 100_000),   # L 57, K 64
        (72, 1, 0, 60_000),     # L 72, K 80
        (90, 1, 0, 60_000),     # L 90, K 96
        (98, 1, 0, 50_000),     # L 98, K 112
        (126, 1, 0, 50_000),    # L 126, K 128
    ]
    with gp.Context(0) as ctx:
        stream = torch.cuda.Stream()
        for order, compress, paf, n in cases:
            L = order // compress
            alpha = np.array([v for v in range(-compress, compress + 1, 2) if compress % 2 == 0 or v != 0],
                             dtype=np.int8)
            seqs = torch.from_numpy(rng.choice(alpha, size=(n, L))).cuda()
            want = torch.zeros((n + 31) // 32, dtype=torch.int32, device="cuda")
            got = torch.full_like(want, -1)
            torch.cuda.synchronize()
            ctx.psd_filter_device(seqs.data_ptr(), n, L, order, paf, gp.GP_PSD_TC_GUARDED, want.data_ptr(),
                                  stream.cuda_stream, stats=True)
            rc = fn(seqs.data_ptr(), n, L, order, paf, got.data_ptr(), stream.cuda_stream)
            assert rc == 0, rc
            torch.cuda.synchronize()
            assert torch.equal(got, want)
            if L <= 57:
                assert int(want.ne(0).sum()) > 0  # the batch does contain passes


def test_noalloc_rejects_batches_over_its_limit():
    torch = pytest.importorskip("torch")
    fn = _entry()
    seqs = torch.zeros((16, 45), dtype=torch.int8, device="cuda")
    mask = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert fn(seqs.data_ptr(), MAX_ROWS + 1, 45, 90, 0, mask.data_ptr(), None) == -1  # GP_ERR_ARG
