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
  reference's own generation functions through oracle/ref_window_driver.cpp,
  and the pair file of the reference's `sort` and `match` over each window's
  candidate files;
* n21_c31/, n27_c31/ -- the sorted, pair and unique files of
  `main N -c 3 1 --paf -2 all` (Legendre-type pairs, odd compression 3 -> 1;
  verbatim), and hashes of the same runs at orders 33 and 39;
* hashes of order 36 at compression 6: the chain 6 -> 3 -> 1 and 6 -> 1;
* manifest.json "n57" -- order 57, paf -2, compression 3 -> 1 in full:
  `gen` over 8 jobs (-n 8 -j 0..7, run in parallel), `sort`, `match`
  (hashes of the sorted files and of the 196,216-line pair file), then the
  uncompression and filter of two 200-line subsets of the pair file (its
  first 200 lines; 200 lines drawn with numpy's default_rng(0), in file
  order).  The reference never reads its line-range options, so each line
  is uncompressed in a directory of its own (one process per line, several
  at a time) and the per-line outputs are concatenated in line order, which
  is what one run over the subset writes; `filter` then runs on each
  subset's concatenated pair file.  About 3 hours on 8 cores; resumable:
  steps whose outputs exist in the work directory are skipped.

Needs the reference sources; run in the build container only:
    python tests/golden/make_golden.py            # everything but n57
    python tests/golden/make_golden.py --windows  # only the window goldens
    python tests/golden/make_golden.py --run=NAME # only the named run (merged)
    python tests/golden/make_golden.py --n57 --workdir DIR  # the order-57 goldens
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
] + [
    # Legendre-type pairs (paf -2) at the odd compression 3 -> 1
    (f"n{n}_c31", [str(n), "-c", "3", "1", "--paf", "-2", "all"],
     [f"{n}-filtered_sorted-a", f"{n}-filtered_sorted-b", f"{n}-pairs-3", f"{n}-pairs-1", f"{n}-unique"], n < 30)
    for n in (21, 27, 33, 39)
] + [
    # compression 6: the chain 6 -> 3 -> 1 (ratio 2 into the odd alphabet, then 3) and 6 -> 1 directly
    ("n36_c631", ["36", "-c", "6", "3", "1", "gen", "sort", "match", "uncompress"],
     ["36-filtered_sorted-a", "36-filtered_sorted-b", "36-pairs-6", "36-pairs-3", "36-pairs-1"], False),
    ("n36_c61", ["36", "-c", "6", "1", "gen", "sort", "match", "uncompress"], ["36-pairs-6", "36-pairs-1"], False),
]
N57_ARGV = ["57", "-c", "3", "1", "--paf", "-2"]
N57_JOBS = 8
N57_HEADS = 200
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
    """The window's candidate files from the reference's own generation
    functions, then the reference's `sort` and `match` over them (the files
    placed as job 0's candidate files of a work directory)."""
    o, c, p, lo, hi = job
    env = dict(os.environ, LC_ALL="C")
    d = os.path.join(tmp, window_key(job).replace("/", "_"))
    wd = os.path.join(d, f"order-{o}")
    os.makedirs(wd)
    fa, fb = os.path.join(wd, f"{o}-filtered-a#0"), os.path.join(wd, f"{o}-filtered-b#0")
    out = subprocess.run([REF_WINDOW_BIN, str(o), str(c), str(p), str(lo), str(hi), fa, fb], check=True,
                         capture_output=True, text=True, env=env).stdout
    rec = {"job": list(job), "necklaces": int(out.split()[-1])}
    for side, path in (("a", fa), ("b", fb)):
        with open(path, "rb") as f:
            rec[side] = {"lines": f.read().count(b"\n"), "sha256": sha256(path)}
    # match returns 1 on an empty input (src/core/match/match_pairs.cpp:32-38), after writing an empty pair file
    r = subprocess.run([REF_BIN, str(o), "-c", str(c), "--paf", str(p), "--dir", d, "sort", "match"], env=env,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    assert r.returncode in (0, 1), (job, r.returncode)
    pairs = os.path.join(wd, f"{o}-pairs-{c}")
    with open(pairs, "rb") as f:
        rec["pairs"] = {"lines": f.read().count(b"\n"), "sha256": sha256(pairs)}
    return rec


def make_windows(manifest):
    sys.path.insert(0, REPO)
    from golaypair_gb300.workloads import batch_windows
    jobs = batch_windows() + batch_windows(1 << 24)
    with tempfile.TemporaryDirectory() as tmp, ThreadPoolExecutor(len(jobs)) as ex:
        recs = list(ex.map(lambda j: run_window(j, tmp), jobs))
    manifest["windows"] = {window_key(r["job"]): r for r in recs}


def n57_subsets(nlines):
    """The two head subsets of the order-57 pair file: line indices (0-based)."""
    import numpy as np
    seeded = sorted(np.random.default_rng(0).choice(nlines, N57_HEADS, replace=False).tolist())
    return {"head200": list(range(N57_HEADS)), "seed200": seeded}


def make_n57(manifest, work, procs):
    env = dict(os.environ, LC_ALL="C")
    full = os.path.join(work, "d")
    wd = os.path.join(full, "order-57")
    if not os.path.exists(os.path.join(wd, "57-pairs-3")):
        ps = [subprocess.Popen([REF_BIN] + N57_ARGV + ["-n", str(N57_JOBS), "-j", str(j), "--dir", full, "gen"],
                               stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env=env)
              for j in range(N57_JOBS)]
        for p in ps:
            assert p.wait() == 0
        for sub in ("sort", "match"):
            subprocess.run([REF_BIN] + N57_ARGV + ["-n", str(N57_JOBS), "--dir", full, sub], check=True, env=env,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    rec = {"argv": N57_ARGV + ["-n", str(N57_JOBS), "gen|sort|match"], "files": {}, "subsets": {}}
    for fn in ("57-filtered_sorted-a", "57-filtered_sorted-b", "57-pairs-3"):
        with open(os.path.join(wd, fn), "rb") as f:
            data = f.read()
        rec["files"][fn] = {"lines": data.count(b"\n"), "sha256": hashlib.sha256(data).hexdigest()}
    with open(os.path.join(wd, "57-pairs-3")) as f:
        lines = f.read().split("\n")[:-1]
    subsets = n57_subsets(len(lines))

    def cost(i):  # expansions of the line's two sides: 3^(entries of magnitude 1, less the first)
        v = lines[i].split()
        return sum(3 ** max(0, sum(1 for x in side if x in ("1", "-1")) - 1) for side in (v[:19], v[19:]))

    todo = sorted(set(i for idx in subsets.values() for i in idx), key=lambda i: -cost(i))

    def one_line(i):  # uncompression of one input line
        d = os.path.join(work, "h", str(i))
        if os.path.exists(os.path.join(d, "ok")):
            return
        os.makedirs(os.path.join(d, "order-57"), exist_ok=True)
        with open(os.path.join(d, "order-57", "57-pairs-3"), "w") as f:
            f.write(lines[i] + "\n")
        subprocess.run([REF_BIN] + N57_ARGV + ["--dir", d, "uncompress"], check=True, env=env,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        for t in ("uncompress_tmp_a", "uncompress_tmp_b", "uncompress_tmp_a.sorted", "uncompress_tmp_b.sorted"):
            os.remove(os.path.join(d, "order-57", t))
        open(os.path.join(d, "ok"), "w").close()

    with ThreadPoolExecutor(procs) as ex:  # longest lines first
        list(ex.map(one_line, todo))
    for name, idx in subsets.items():
        d = os.path.join(work, name)
        os.makedirs(os.path.join(d, "order-57"), exist_ok=True)
        with open(os.path.join(d, "order-57", "57-pairs-3"), "w") as f:
            f.write("".join(lines[i] + "\n" for i in idx))
        with open(os.path.join(d, "order-57", "57-pairs-1"), "wb") as f:
            for i in idx:
                with open(os.path.join(work, "h", str(i), "order-57", "57-pairs-1"), "rb") as g:
                    f.write(g.read())
        if not os.path.exists(os.path.join(d, "order-57", "57-unique")):
            subprocess.run([REF_BIN] + N57_ARGV + ["--dir", d, "filter"], check=True, env=env,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        srec = {"indices": idx, "files": {}}
        for fn in ("57-pairs-1", "57-unique"):
            with open(os.path.join(d, "order-57", fn), "rb") as f:
                data = f.read()
            srec["files"][fn] = {"lines": data.count(b"\n"), "sha256": hashlib.sha256(data).hexdigest()}
        rec["subsets"][name] = srec
    manifest["n57"] = rec


def arg_value(name, default=None):
    for i, a in enumerate(sys.argv[1:], 1):
        if a.startswith(name + "="):
            return a.split("=", 1)[1]
        if a == name and i + 1 < len(sys.argv):
            return sys.argv[i + 1]
    return default


def main():
    subprocess.run(["bash", os.path.join(REPO, "oracle", "build_ref.sh")], check=True)
    if not os.path.exists(REF_BIN):
        sys.exit("reference binary missing (no reference sources here)")
    if "--n57" in sys.argv[1:]:
        work = os.path.abspath(arg_value("--workdir") or tempfile.mkdtemp(prefix="golden57_"))
        procs = int(arg_value("--procs", str(N57_JOBS)))
        manifest = {}
        make_n57(manifest, work, procs)
        with open(os.path.join(HERE, "manifest.json")) as f:  # merged into the current manifest at the end
            cur = json.load(f)
        cur["n57"] = manifest["n57"]
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(cur, f, indent=1, sort_keys=True)
        print("order-57 goldens written")
        return
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
