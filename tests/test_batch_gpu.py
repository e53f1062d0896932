"""Batched generation (gp_generate_batch): several orders / compressions of
different lengths in one engine run, one enumerator launch per iteration
and a replayed CUDA graph.

Bar: every job's A and B files are byte-identical to those of the
reference (golden hashes) or of the oracle over the same word window, and
do not depend on the engine's settings (graph or direct launches, soft
capacity, enumerator variant, windows per thread, filter grid, one launch
per kernel over all jobs or per-job launches, tuner).
"""
import ctypes
import hashlib
import os
import subprocess

import pytest

import golaypair_gb300 as gp
from conftest import GenStats, read

pytestmark = pytest.mark.gpu

# (order, compress, paf, begin, end): lengths 8, 17, 19, 25, 29, 18
JOBS = [
    (16, 2, 0, 0, 3 ** 8),                          # whole space
    (34, 2, 0, 0, 3 ** 17),                         # whole space (golden hashes)
    (57, 3, -2, 0, 1 << 23),
    (50, 2, 0, 123456789012, 123456789012 + (1 << 24)),
    (58, 2, 0, 31415926535897, 31415926535897 + (1 << 22)),
    (90, 5, 0, 98765432109876, 98765432109876 + (1 << 22)),
]


def run_batch(ctx, tmp, tag, jobs=JOBS, **kw):
    spec = []
    for i, (o, c, p, lo, hi) in enumerate(jobs):
        spec.append((o, c, p, lo, hi, tmp / f"{tag}{i}a", tmp / f"{tag}{i}b"))
    cfg = gp.BatchConfig()
    autotune = kw.pop("autotune", False)
    for k, v in kw.items():
        setattr(cfg, k, v)
    stats, cfg = ctx.generate_batch(spec, autotune=autotune, config=cfg)
    files = [(read(a), read(b)) for (_, _, _, _, _, a, b) in spec]
    return files, stats, cfg


@pytest.fixture(scope="module")
def default_run(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("batch")
    with gp.Context(0) as ctx:
        return run_batch(ctx, tmp, "d")


def test_batch_matches_reference_and_oracle(default_run, oracle_lib, golden_manifest, tmp_path):
    files, stats, cfg = default_run
    assert cfg.iterations >= 1
    for i, (o, c, p, lo, hi) in enumerate(JOBS):
        ga, gb = files[i]
        if (o, c) == (34, 2):
            meta = golden_manifest["runs"]["n34"]["files"]
            assert hashlib.sha256(ga).hexdigest() == meta["34-filtered-a#0"]["sha256"]
            assert hashlib.sha256(gb).hexdigest() == meta["34-filtered-b#0"]["sha256"]
            continue
        oa, ob = str(tmp_path / f"o{i}a"), str(tmp_path / f"o{i}b")
        ost = GenStats()
        oracle_lib.gpo_generate_window(o, c, p, oa.encode(), ob.encode(), lo >> 64, lo & (2**64 - 1), hi >> 64,
                                       hi & (2**64 - 1), ctypes.byref(ost))
        assert ga == read(oa), (o, c)
        assert gb == read(ob), (o, c)
        assert stats[i].necklaces == ost.necklaces, (o, c)
        assert stats[i].written_a + stats[i].written_b == ga.count(b"\n") + gb.count(b"\n")


def test_batch_equals_single_windows(default_run, tmp_path):
    files, stats, _ = default_run
    with gp.Context(0) as ctx:
        for i, (o, c, p, lo, hi) in enumerate(JOBS):
            st = ctx.generate_window(o, c, p, lo, hi, tmp_path / "a", tmp_path / "b")
            assert (read(tmp_path / "a"), read(tmp_path / "b")) == files[i], (o, c)
            for f in ("necklaces", "candidates", "psd_pass", "written_a", "written_b"):
                assert getattr(st, f) == getattr(stats[i], f), (o, c, f)


@pytest.mark.parametrize("settings", [
    {"no_graph": 1},
    {"cand_cap": 1 << 16},                   # many iterations: windows left and resumed
    {"cand_cap": 5000, "no_graph": 1},
    {"enum_variant": 1},
    {"enum_variant": 2},
    {"windows_per_thread": 4},
    {"tc_ctas_per_sm": 1},
    {"multi_launch": 1},                     # one launch per kernel over all jobs (K = 16 and 32 tiles)
    {"multi_launch": 1, "no_graph": 1},
    {"multi_launch": 1, "cand_cap": 5000},
    {"multi_launch": 1, "tc_ctas_per_sm": 1},
])
def test_batch_settings_do_not_change_results(default_run, tmp_path, settings):
    files, stats, _ = default_run
    with gp.Context(0) as ctx:
        got, st2, cfg = run_batch(ctx, tmp_path, "s", **settings)
    assert got == files
    for a, b in zip(stats, st2):
        assert (a.necklaces, a.candidates, a.psd_pass) == (b.necklaces, b.candidates, b.psd_pass)
    if "cand_cap" in settings:
        assert cfg.iterations > 1
    assert cfg.multi_launch == settings.get("multi_launch", 0)


def test_batch_multi_launch_at_k64(tmp_path):
    """One filter launch over rows of lengths 17, 19 (K = 32 tiles) and 50
    (K = 64 tiles, the one-CTA-per-SM instance) gives the files of per-job
    launches."""
    jobs = [(34, 2, 0, 0, 3 ** 17), (100, 2, 0, 271828182845904523, 271828182845904523 + (1 << 24)),
            (57, 3, -2, 1 << 30, (1 << 30) + (1 << 22))]
    with gp.Context(0) as ctx:
        per_job, st1, _ = run_batch(ctx, tmp_path, "p", jobs=jobs)
        multi, st2, cfg = run_batch(ctx, tmp_path, "m", jobs=jobs, multi_launch=1, cand_cap=1 << 18)
    assert cfg.multi_launch == 1 and cfg.iterations > 1
    assert multi == per_job
    for a, b in zip(st1, st2):
        assert (a.necklaces, a.candidates, a.psd_pass) == (b.necklaces, b.candidates, b.psd_pass)
    assert sum(len(a) + len(b) for a, b in multi) > 0


def test_batch_multi_launch_rejects_long_rows(tmp_path):
    """Rows of length 68 need K = 80, beyond the multi-job filter (K <= 64): asking
    for one launch is an error, the per-job engine runs them."""
    jobs = [(68, 1, 0, 0, 1 << 20), (34, 2, 0, 0, 1 << 20)]
    with gp.Context(0) as ctx:
        with pytest.raises(gp.GPError):
            run_batch(ctx, tmp_path, "r", jobs=jobs, multi_launch=1)
        _, _, cfg = run_batch(ctx, tmp_path, "q", jobs=jobs)
        assert cfg.multi_launch == 0


def test_batch_autotune_is_cached_and_exact(default_run, tmp_path):
    files, _, _ = default_run
    with gp.Context(0) as ctx:
        got, _, cfg = run_batch(ctx, tmp_path, "t", autotune=True)
        assert got == files
        assert cfg.enum_variant in (0, 1, 2) and cfg.windows_per_thread in (1, 4)
        assert cfg.tc_ctas_per_sm in (0, 1) and cfg.no_graph == 0
        assert cfg.tune_seconds > 0
        got2, _, cfg2 = run_batch(ctx, tmp_path, "u", autotune=True)
        assert got2 == files
        assert cfg2.tune_seconds == 0
        assert (cfg2.enum_variant, cfg2.windows_per_thread, cfg2.cand_cap) == (
            cfg.enum_variant, cfg.windows_per_thread, cfg.cand_cap)


def test_batch_rejects_bad_jobs(tmp_path):
    with gp.Context(0) as ctx:
        with pytest.raises(gp.GPError):
            ctx.generate_batch([(15, 2, 0, 0, 10, tmp_path / "a", tmp_path / "b")])  # 15 not divisible by 2
        with pytest.raises(gp.GPError):
            ctx.generate_batch([(16, 2, 0, 0, 10, tmp_path / "a", tmp_path / "b")] * 9)  # more than 8 jobs


@pytest.mark.parametrize("size,multi", [(1 << 24, 0), (1 << 24, 1), (1 << 32, None)])
def test_uneven_batch_windows_match_reference(golden_manifest, tmp_path, size, multi):
    """The uneven batch (orders 34, 50, 58, 68 at compression 2, 90 at
    compression 5) over its seed-chosen windows, against the reference's own
    generation functions run over the same windows (the bench's workload at
    2^32 words): per-job launches, one launch per kernel over all jobs
    (K = 32 and 48 tiles), and the tuner's choice."""
    from golaypair_gb300.workloads import batch_windows
    wins = batch_windows(size)
    recs = golden_manifest["windows"]
    kw = {"autotune": True} if multi is None else {"multi_launch": multi}
    with gp.Context(0) as ctx:
        files, stats, cfg = run_batch(ctx, tmp_path, "w", jobs=wins, **kw)
    if multi is not None:
        assert cfg.multi_launch == multi
    for i, (w, (a, b), st) in enumerate(zip(wins, files, stats)):
        rec = recs["%d/%d/%d/%d-%d" % tuple(w)]
        assert st.necklaces == rec["necklaces"], w
        assert a.count(b"\n") == rec["a"]["lines"] and b.count(b"\n") == rec["b"]["lines"], w
        assert hashlib.sha256(a).hexdigest() == rec["a"]["sha256"], w
        assert hashlib.sha256(b).hexdigest() == rec["b"]["sha256"], w
        if "pairs" not in rec:
            continue
        # the per-order pair set: sort and match over the batch's files, as the
        # reference's sort and match ran over its own window files
        o, c, p = w[0], w[1], w[2]
        wd = tmp_path / f"pairs{i}" / f"order-{o}"
        wd.mkdir(parents=True)
        (wd / f"{o}-filtered-a#0").write_bytes(a)
        (wd / f"{o}-filtered-b#0").write_bytes(b)
        r = subprocess.run([gp.CLI_PATH, str(o), "-c", str(c), "--paf", str(p), "--dir", str(wd.parent), "sort",
                            "match"], capture_output=True, text=True, env=dict(os.environ, LC_ALL="C"))
        assert r.returncode in (0, 1), r.stderr
        pairs = read(str(wd / f"{o}-pairs-{c}"))
        assert pairs.count(b"\n") == rec["pairs"]["lines"], w
        assert hashlib.sha256(pairs).hexdigest() == rec["pairs"]["sha256"], w
