"""Checkpointed generation: a search stopped every few pipeline iterations
and resumed from its checkpoint file ends with the same A and B files as an
uninterrupted run -- byte for byte the reference's own output on the
uneven batch's order-58 window -- and leaves no checkpoint behind."""
import ctypes
import hashlib
import os
import subprocess

import pytest

import golaypair_gb300 as gp
from conftest import read

pytestmark = pytest.mark.gpu


def test_window_resumes_to_reference_files(golden_manifest, tmp_path):
    from golaypair_gb300.workloads import batch_windows
    w = [x for x in batch_windows() if x[0] == 58][0]  # 2^32 words, ~60 iterations
    rec = golden_manifest["windows"]["%d/%d/%d/%d-%d" % tuple(w)]
    o, c, p, lo, hi = w
    ck = tmp_path / "ck"
    calls = 0
    with gp.Context(0) as ctx:
        while True:
            done, st = ctx.generate_window_resumable(o, c, p, lo, hi, tmp_path / "a", tmp_path / "b", ck,
                                                     max_iterations=7)
            calls += 1
            assert calls < 100
            if done:
                break
            assert ck.exists() and not (tmp_path / "a").exists()
    assert calls > 2
    assert not ck.exists()
    assert st.necklaces == rec["necklaces"]
    a, b = read(tmp_path / "a"), read(tmp_path / "b")
    assert hashlib.sha256(a).hexdigest() == rec["a"]["sha256"]
    assert hashlib.sha256(b).hexdigest() == rec["b"]["sha256"]


def test_shard_resumes_to_uninterrupted_files(tmp_path):
    """Job 3 of 8 of order 57 (paf -2, compression 3): stopped every 10
    iterations, against gp_generate of the same job in one call."""
    with gp.Context(0) as ctx:
        st0 = gp.GenStats()
        ctx.check(ctx._lib.gp_generate(ctx.handle, 57, 3, -2, 3, 8, str(tmp_path / "fa").encode(),
                                       str(tmp_path / "fb").encode(), ctypes.byref(st0)), "gp_generate")
        done = ctypes.c_int(0)
        st = gp.GenStats()
        calls = 0
        while not done.value:
            ctx.check(ctx._lib.gp_generate_resumable(ctx.handle, 57, 3, -2, 3, 8, str(tmp_path / "ra").encode(),
                                                     str(tmp_path / "rb").encode(), str(tmp_path / "ck").encode(), 10,
                                                     0.0, ctypes.byref(done), ctypes.byref(st)),
                      "gp_generate_resumable")
            calls += 1
            assert calls < 200
    assert calls > 1
    assert read(tmp_path / "ra") == read(tmp_path / "fa")
    assert read(tmp_path / "rb") == read(tmp_path / "fb")
    assert (st.necklaces, st.candidates, st.psd_pass) == (st0.necklaces, st0.candidates, st0.psd_pass)


def test_checkpoint_of_another_job_is_rejected(tmp_path):
    from golaypair_gb300.workloads import batch_windows
    o, c, p, lo, hi = [x for x in batch_windows() if x[0] == 58][0]
    ck = tmp_path / "ck"
    with gp.Context(0) as ctx:
        done, _ = ctx.generate_window_resumable(o, c, p, lo, hi, tmp_path / "a", tmp_path / "b", ck, max_iterations=1)
        assert not done and ck.exists()
        with pytest.raises(gp.GPError, match="another job"):
            ctx.generate_window_resumable(o, c, p, lo + 1, hi, tmp_path / "a", tmp_path / "b", ck, max_iterations=1)


def test_cli_gen_with_checkpoint_matches_reference(golden_manifest, tmp_path):
    """golay 34 -c 2 gen --checkpoint FILE: finishes in one call here (few
    candidates), exit code 0, the reference's files, no checkpoint left."""
    meta = golden_manifest["runs"]["n34"]["files"]
    ck = tmp_path / "ck"
    r = subprocess.run([gp.CLI_PATH, "34", "-c", "2", "--dir", str(tmp_path), "gen", "--checkpoint", str(ck),
                        "--max-iterations", "1"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       env=dict(os.environ, LC_ALL="C"))
    assert r.returncode == 0, r.stderr
    assert not ck.exists()
    wd = tmp_path / "order-34"
    for fn, m in meta.items():
        assert hashlib.sha256(read(wd / fn)).hexdigest() == m["sha256"], fn
