"""Failures injected on the host (no GPU fault): an unusable work
directory, missing arguments.  The driver must report them and exit non-zero
before touching the GPU."""
import subprocess

import golaypair_gb300 as gp


def run(args):
    return subprocess.run([gp.CLI_PATH] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)


def test_unwritable_work_directory(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("not a directory")
    r = run(["26", "-c", "2", "--dir", str(blocker / "sub"), "gen"])
    assert r.returncode == 1
    assert "Failed to create temp directories" in r.stderr


def test_missing_order_and_subcommand():
    r = run(["gen"])
    assert r.returncode != 0 and "order is required" in r.stderr
    r = run(["26"])
    assert r.returncode != 0 and "subcommand is required" in r.stderr
