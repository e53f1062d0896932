"""Binary survivor files from the GPU generation: `gen --binary` writes them,
`sort` reads them directly and `export` turns them into text; every file
that reaches the reference's format is byte-identical to the reference's."""
import hashlib
import os
import subprocess

import pytest

import golaypair_gb300 as gp
from conftest import GOLDEN, read

pytestmark = pytest.mark.gpu
ENV = dict(os.environ, LC_ALL="C")
MAGIC = b"GPSURV01"


def golay(args, d):
    r = subprocess.run([gp.CLI_PATH] + args[:3] + ["--dir", str(d)] + args[3:], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, env=ENV)
    assert r.returncode == 0, r.stderr + r.stdout
    return r


def sha(path):
    return hashlib.sha256(read(path)).hexdigest()


def test_n26_binary_gen_sort_match_export(tmp_path, golden_manifest):
    files = golden_manifest["runs"]["n26"]["files"]
    wd = tmp_path / "order-26"
    golay(["26", "-c", "2", "gen", "--binary"], tmp_path)
    for ab in "ab":
        raw = read(wd / f"26-filtered-{ab}#0")
        assert raw[:8] == MAGIC
        assert len(raw) < len(read(os.path.join(GOLDEN, "n26", f"26-filtered-{ab}_0")))
    # sort reads the binary files directly
    golay(["26", "-c", "2", "sort", "match"], tmp_path)
    for fn in ("26-filtered_sorted-a", "26-filtered_sorted-b", "26-pairs-2"):
        assert sha(wd / fn) == files[fn]["sha256"], fn
    golay(["26", "-c", "2", "export"], tmp_path)
    for ab in "ab":
        fn = f"26-filtered-{ab}#0"
        assert sha(wd / fn) == files[fn]["sha256"], fn


def test_n34_binary_gen_exports_reference_files(tmp_path, golden_manifest):
    files = golden_manifest["runs"]["n34"]["files"]
    wd = tmp_path / "order-34"
    golay(["34", "-c", "2", "gen", "--binary"], tmp_path)
    sizes = {ab: os.path.getsize(wd / f"34-filtered-{ab}#0") for ab in "ab"}
    golay(["34", "-c", "2", "export"], tmp_path)
    for ab in "ab":
        fn = f"34-filtered-{ab}#0"
        assert sha(wd / fn) == files[fn]["sha256"], fn
        assert sizes[ab] * 3 < os.path.getsize(wd / fn)


def test_window_binary_equals_text_call(tmp_path, golden_manifest):
    """Python API: the order-58 window of the uneven batch written as binary
    and exported equals the reference's files for that window."""
    from golaypair_gb300.workloads import batch_windows
    w = [x for x in batch_windows() if x[0] == 58][0]
    rec = golden_manifest["windows"]["%d/%d/%d/%d-%d" % tuple(w)]
    o, c, p, lo, hi = w
    with gp.Context(0) as ctx:
        ctx.set_output_format(gp.GP_FORMAT_BINARY)
        st = ctx.generate_window(o, c, p, lo, hi, tmp_path / "a.bin", tmp_path / "b.bin")
    assert st.necklaces == rec["necklaces"]
    for ab in "ab":
        gp.export_text(tmp_path / f"{ab}.bin", tmp_path / f"{ab}.txt")
        assert sha(tmp_path / f"{ab}.txt") == rec[ab]["sha256"]
