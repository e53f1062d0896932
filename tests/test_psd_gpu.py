"""Parity of the batched PSD filter (both arithmetic modes) with the oracle.

Bar: verdicts bit-exact against the oracle's FP64 filter (which restates
src/utils/fourier.cpp:25-52).  The tensor-core mode's fp32 PSD error against
FP64 must stay below its guard band: |PSD_tc - PSD_fp64| < 1e-3 * 2n.
"""
import itertools

import numpy as np
import pytest

import golaypair_gb300 as gp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    with gp.Context(0) as c:
        yield c


def alphabet(c):
    if c % 2 == 0:
        return list(range(-c, c + 1, 2))
    return [v for v in range(-c, c + 1, 2)]


def oracle_verdicts(oracle_lib, seqs, order, paf):
    seqs = np.ascontiguousarray(seqs, dtype=np.int8)
    v = np.zeros(len(seqs), dtype=np.uint8)
    oracle_lib.gpo_psd_filter_batch(seqs.ctypes.data, len(seqs), seqs.shape[1], order, paf, v.ctypes.data, 8)
    return v.astype(bool)


CASES = [  # (order, compress, paf)
    (16, 2, 0), (26, 2, 0), (34, 2, 0), (50, 2, 0), (58, 2, 0), (68, 2, 0), (90, 2, 0), (90, 5, 0),
    (57, 3, -2), (57, 1, -2), (16, 1, 0), (26, 1, 0), (38, 1, 0), (98, 1, 0), (126, 1, 0), (252, 2, 0),
    (70, 1, 0), (86, 1, 0), (170, 2, 0),  # padded lengths K = 80 and 96
    # int8 rows of a length not a multiple of 4 are read from the 4-byte
    # boundary below them and placed 1-3 columns along when L + max shift
    # <= K (K <= 64): L = 46 fills K = 48 exactly; L = 31, 47, 63 (L + 3 > K)
    # keep the byte-realigning loads; L = 54, 60 at K = 64
    (92, 2, 0), (62, 2, 0), (94, 2, 0), (126, 2, 0), (54, 1, 0), (60, 1, 0),
]


@pytest.mark.parametrize("order,compress,paf", CASES)
@pytest.mark.parametrize("mode", [gp.GP_PSD_FP64, gp.GP_PSD_TC_GUARDED])
def test_psd_filter_random_matches_oracle(ctx, oracle_lib, order, compress, paf, mode):
    L = order // compress
    rng = np.random.default_rng(order * 7 + compress)
    n = 50_000 + 77  # tail tile and partial mask word
    seqs = rng.choice(np.array(alphabet(compress), dtype=np.int8), size=(n, L))
    got, st = ctx.psd_filter(seqs, order, paf, mode)
    want = oracle_verdicts(oracle_lib, seqs, order, paf)
    assert np.array_equal(got, want), f"{np.sum(got != want)} verdicts differ"
    assert st.n_pass == want.sum()


def _words(L, alpha):
    return np.array(list(itertools.product(alpha, repeat=L)), dtype=np.int8)


@pytest.mark.parametrize("mode", [gp.GP_PSD_FP64, gp.GP_PSD_TC_GUARDED])
def test_psd_filter_exhaustive_n16_has_bound_ties(ctx, oracle_lib, mode):
    """All 3^8 words of order 16 / compress 2: many PSD values equal the bound
    32 exactly and pass only through the +0.001 slack."""
    seqs = _words(8, [-2, 0, 2])
    got, _ = ctx.psd_filter(seqs, 16, 0, mode)
    assert np.array_equal(got, oracle_verdicts(oracle_lib, seqs, 16, 0))


@pytest.mark.parametrize("mode", [gp.GP_PSD_FP64, gp.GP_PSD_TC_GUARDED])
def test_psd_filter_exhaustive_n26(ctx, oracle_lib, mode):
    seqs = _words(13, [-2, 0, 2])  # 1,594,323 words
    got, _ = ctx.psd_filter(seqs, 26, 0, mode)
    assert np.array_equal(got, oracle_verdicts(oracle_lib, seqs, 26, 0))


def test_psd_filter_cfg4_distribution(ctx, oracle_lib):
    """Synthetic throughput workload shape: length 45 over {-2,0,2}, row sums
    with square in {a^2 : a^2 + b^2 = 180} = {36, 144}."""
    rng = np.random.default_rng(0)
    L = 45
    out = []
    while sum(len(o) for o in out) < 400_000:
        s = rng.choice(np.array([-2, 0, 2], dtype=np.int8), size=(400_000, L))
        rs = s.astype(np.int32).sum(1)
        out.append(s[np.isin(rs, [-12, -6, 6, 12])])
    seqs = np.concatenate(out)[:400_000]
    for mode in (gp.GP_PSD_FP64, gp.GP_PSD_TC_GUARDED):
        got, st = ctx.psd_filter(seqs, 90, 0, mode)
        assert np.array_equal(got, oracle_verdicts(oracle_lib, seqs, 90, 0))
    assert st.n_unsure < 0.01 * len(seqs)


@pytest.mark.parametrize("order,compress,paf", [(16, 2, 0), (26, 2, 0), (57, 3, -2), (90, 2, 0), (90, 5, 0),
                                                (57, 1, -2), (126, 1, 0), (62, 2, 0), (92, 2, 0)])
def test_tc_psd_error_within_guard(ctx, oracle_lib, order, compress, paf):
    L = order // compress
    rng = np.random.default_rng(5)
    seqs = rng.choice(np.array(alphabet(compress), dtype=np.int8), size=(20_000, L))
    tc = ctx.psd_tc_values(seqs).astype(np.float64)
    ref = ctx.psd_fp64_values(seqs)[:, 1:L // 2 + 1]
    err = np.abs(tc - ref).max()
    guard = 1e-3 * 2 * order
    print(f"order {order} c {compress}: max |PSD_fp32 - PSD_fp64| = {err:.3e} (guard {guard:.3g})")
    assert err < guard / 10


def test_fp64_values_match_oracle(ctx, oracle_lib):
    import ctypes
    rng = np.random.default_rng(3)
    for L in (8, 13, 19, 45, 57):
        seqs = rng.choice(np.array([-3, -1, 1, 3], dtype=np.int8), size=(64, L))
        got = ctx.psd_fp64_values(seqs)
        psd = (ctypes.c_double * L)()
        for i in range(64):
            s = (ctypes.c_int * L)(*seqs[i].tolist())
            oracle_lib.gpo_psd(s, L, psd)
            assert np.allclose(got[i], np.array(psd[:]), rtol=0, atol=1e-9)


def test_bounded_wait_gives_up_and_context_stays_usable(ctx, oracle_lib):
    """Failure detection without a GPU fault: a device wait on a barrier that
    nothing completes gives up after its limit and reports GP_ERR_TIMEOUT;
    the same context then filters correctly."""
    import time
    t0 = time.time()
    rc = ctx._lib.gp_debug_wait_timeout(ctx.handle, 50_000_000)  # 50 ms
    assert rc == -3  # GP_ERR_TIMEOUT
    assert time.time() - t0 < 5
    assert b"timed out" in ctx._lib.gp_last_error(ctx.handle)
    seqs = np.array(list(itertools.product([-2, 0, 2], repeat=8)), dtype=np.int8)
    want = np.zeros(len(seqs), dtype=np.uint8)
    oracle_lib.gpo_psd_filter_batch(seqs.ctypes.data, len(seqs), 8, 16, 0, want.ctypes.data, 1)
    got, _ = ctx.psd_filter(seqs, 16, 0, gp.GP_PSD_TC_GUARDED)
    assert np.array_equal(got.astype(bool), want.astype(bool))


@pytest.mark.parametrize("L", [45, 47])
def test_device_rows_at_any_byte_offset(ctx, oracle_lib, L):
    """gp_psd_filter_device on rows that start at byte offsets 0, 16 (whole
    tiles bulk-copied; length 45 takes the shifted loads, 47 the
    byte-realigning ones) and 1, 3, 45 (not 16-byte aligned: every row read
    by plain loads); the verdicts equal the oracle's in every case."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(L)
    n = 20_000 + 45  # a tail tile and a partial mask word
    seqs = rng.choice(np.array([-2, 0, 2], dtype=np.int8), size=(n, L))
    want = oracle_verdicts(oracle_lib, seqs, 2 * L, 0)
    flat = torch.from_numpy(seqs.reshape(-1))
    for off in (0, 16, 1, 3, 45):
        buf = torch.zeros(n * L + 64, dtype=torch.int8, device="cuda")
        buf[off:off + n * L] = flat.cuda()
        mask = torch.full(((n + 31) // 32,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ctx.psd_filter_device(buf.data_ptr() + off, n, L, 2 * L, 0, gp.GP_PSD_TC_GUARDED, mask.data_ptr(), None)
        ctx.check_stream(None)
        bits = mask.cpu().numpy().view(np.uint32)
        got = ((bits[np.arange(n) // 32] >> (np.arange(n) % 32)) & 1).astype(bool)
        assert np.array_equal(got, want), f"offset {off}: {np.sum(got != want)} verdicts differ"
