#!/usr/bin/env python3
"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Builds the reference's own C++ sources (oracle/build_ref.sh, stand-in FFTW and
Boost headers) into oracle/_ref/golay_ref, runs it under LC_ALL=C, and stores:

* n16/, n26/   -- every stage file of `main N -c 2 1 all` (small, verbatim);
* manifest.json -- line counts and SHA-256 of those files, plus of the larger
  outputs that are not stored verbatim (n=34 gen, the n=57 lambda=-2 c=3
  shard 7 of 1000);
* manifest.json "windows" -- the same for the uneven batch's windows
  (golaypair_gb300/workloads.py) at 2^32 and 2^24 words, produced by the
  reference's own generation functions through oracle/ref_window_driver.cpp.

Needs the reference sources; run in the build container only:
    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py --windows  # only the window goldens
    python tests/golden/make_golden.py --run=NAME # only the named run (merged)
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(REPO, "oracle", "_ref", "golay_ref")
REF_WINDOW_BIN = os.path.join(REPO, "oracle", "_ref", "golay_ref_window")

# (name, argv after the binary, files to record, keep verbatim)
RUNS = [
    ("n16", ["16", "-c", "2", "1", "all"],
     ["16-filtered-a#0", "16-filtered-b#0", "16-filtered_sorted-a", "16-filtered_sorted-b",
      "16-pairs-2", "16-pairs-1", "16-unique"], True),
    ("n26", ["26", "-c", "2", "1", "all"],
     ["26-filtered-a#0", "26-filtered-b#0", "26-filtered_sorted-a", "26-filtered_sorted-b",
      "26-pairs-2", "26-pairs-1", "26-unique"], True),
    ("n34", ["34", "-c", "2", "gen"], ["34-filtered-a#0", "34-filtered-b#0"], False),
    ("n57_shard7of1000", ["57", "-c", "3", "1", "--paf", "-2", "-n", "1000", "-j", "7", "gen"],
     ["57-filtered-a#7", "57-filtered-b#7"], False),
    # a three-level chain: generation at compression 4, uncompression 4 -> 2 -> 1
    ("n32_c421", ["32", "-c", "4", "2", "1", "gen", "sort", "match", "uncompress"],
     ["32-filtered-a#0", "32-filtered-b#0", "32-filtered_sorted-a", "32-filtered_sorted-b", "32-pairs-4",
      "32-pairs-2", "32-pairs-1"], False),
]
SUBCOMMANDS = {"gen", "sort", "match", "uncompress", "filter", "all"}


def split_argv(args):
    """(options and positionals, subcommands): --dir goes between them."""
    i = len(args)
    while i > 0 and args[i - 1] in SUBCOMMANDS:
        i -= 1
    return args[:i], args[i:]


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def window_key(job):
    return "%d/%d/%d/%d-%d" % tuple(job)


def run_window(job, tmp):
    o, c, p, lo, hi = job
    fa, fb = os.path.join(tmp, window_key(job).replace("/", "_") + "a"), os.path.join(tmp, window_key(job).replace("/", "_") + "b")
    out = subprocess.run([REF_WINDOW_BIN, str(o), str(c), str(p), str(lo), str(hi), fa, fb], check=True,
                         capture_output=True, text=True, env=dict(os.environ, LC_ALL="C")).stdout
    rec = {"job": list(job), "necklaces": int(out.split()[-1])}
    for side, path in (("a", fa), ("b", fb)):
        with open(path, "rb") as f:
            rec[side] = {"lines": f.read().count(b"\n"), "sha256": sha256(path)}
    return rec


def make_windows(manifest):
    sys.path.insert(0, REPO)
    from golaypair_gb300.workloads import batch_windows
    jobs = batch_windows() + batch_windows(1 << 24)
    with tempfile.TemporaryDirectory() as tmp, ThreadPoolExecutor(len(jobs)) as ex:
        recs = list(ex.map(lambda j: run_window(j, tmp), jobs))
    manifest["windows"] = {window_key(r["job"]): r for r in recs}


def main():
    subprocess.run(["bash", os.path.join(REPO, "oracle", "build_ref.sh")], check=True)
    if not os.path.exists(REF_BIN):
        sys.exit("reference binary missing (no reference sources here)")
    if "--windows" in sys.argv[1:]:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
        make_windows(manifest)
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1, sort_keys=True)
        print("window goldens written")
        return
    env = dict(os.environ, LC_ALL="C")
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--run=")]
    if only:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
    else:
        manifest = {"generator": "reference sources built by oracle/build_ref.sh, LC_ALL=C", "runs": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, args, files, keep in RUNS:
            if only and name not in only:
                continue
            d = os.path.join(tmp, name)
            opts, subs = split_argv(args)
            subprocess.run([REF_BIN] + opts + ["--dir", d] + subs, check=True, env=env,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            order = args[0]
            wd = os.path.join(d, f"order-{order}")
            rec = {"argv": args, "files": {}}
            for fn in files:
                p = os.path.join(wd, fn)
                with open(p, "rb") as f:
                    nlines = f.read().count(b"\n")
                rec["files"][fn] = {"lines": nlines, "sha256": sha256(p)}
                if keep:
                    os.makedirs(os.path.join(HERE, name), exist_ok=True)
                    shutil.copy(p, os.path.join(HERE, name, fn.replace("#", "_")))
            manifest["runs"][name] = rec
    if not only:
        make_windows(manifest)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
