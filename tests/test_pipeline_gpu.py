"""End-to-end parity of the GPU pipeline (the `golay` driver, i.e. the C ABI
stage by stage) with the reference's own outputs and with the oracle.

Bar: byte-identical files (candidate files, sorted files, pair files,
unique pairs) against the golden fixtures produced by the reference, and
against the oracle for cases the fixtures do not cover.
"""
import ctypes
import hashlib
import os
import subprocess

import numpy as np
import pytest

import golaypair_gb300 as gp
from conftest import GOLDEN, GenStats, read

pytestmark = pytest.mark.gpu
ENV = dict(os.environ, LC_ALL="C")


SUBCOMMANDS = {"gen", "sort", "match", "uncompress", "filter", "all"}


def golay(args, tmp, check=True):
    """Runs the golay driver with --dir before the first subcommand (global
    options precede subcommands)."""
    d = str(tmp)
    i = next((k for k, a in enumerate(args) if a in SUBCOMMANDS), len(args))
    argv = [gp.CLI_PATH] + args[:i] + ["--dir", d] + args[i:]
    r = subprocess.run(argv, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=ENV)
    if check:
        assert r.returncode == 0, r.stderr + r.stdout
    return r, os.path.join(d, f"order-{args[0]}")


@pytest.mark.parametrize("name", ["n16", "n26", "n21_c31", "n27_c31"])
def test_all_matches_reference(tmp_path, golden_manifest, name):
    rec = golden_manifest["runs"][name]
    _, wd = golay(rec["argv"], tmp_path)
    for fn in rec["files"]:
        got = read(os.path.join(wd, fn))
        want = read(os.path.join(GOLDEN, name, fn.replace("#", "_")))
        assert got == want, fn


@pytest.mark.parametrize("name", ["n34", "n57_shard7of1000", "n32_c421", "n33_c31", "n39_c31", "n36_c631", "n36_c61"])
def test_gen_matches_reference_hash(tmp_path, golden_manifest, name):
    """Hashes of the reference's own outputs; n32_c421 runs generation at
    compression 4 and uncompresses 4 -> 2 -> 1 (90,320 pairs at length 32);
    n33_c31 and n39_c31 run the whole pipeline for Legendre-type pairs at
    compression 3 -> 1 (9,370 pairs of length 39, 2,318 classes); n36_c631
    uncompresses order 36 from compression 6 to 3 (2,309 pairs over the
    alphabet +-1, +-3) and on to 1, n36_c61 from 6 to 1 directly (up to 20
    partitions per entry)."""
    rec = golden_manifest["runs"][name]
    r, wd = golay(rec["argv"], tmp_path)
    for fn, meta in rec["files"].items():
        got = read(os.path.join(wd, fn))
        assert got.count(b"\n") == meta["lines"], fn
        assert hashlib.sha256(got).hexdigest() == meta["sha256"], fn


@pytest.mark.parametrize("order,compress,paf,lo,size", [
    (50, 2, 0, 123456789012, 1 << 24),      # length 25 over {-2,0,2}
    (58, 2, 0, 31415926535897, 1 << 22),    # length 29
    (90, 5, 0, 98765432109876, 1 << 22),    # length 18 over {-5..5 odd}
    (57, 3, -2, 0, 1 << 23),                # length 19, window at the start
])
def test_window_matches_oracle(oracle_lib, tmp_path, order, compress, paf, lo, size):
    hi = lo + size
    with gp.Context(0) as ctx:
        st = gp.GenStats()
        ga, gb = str(tmp_path / "ga"), str(tmp_path / "gb")
        ctx.check(ctx._lib.gp_generate_window(ctx.handle, order, compress, paf, lo >> 64, lo & (2**64 - 1), hi >> 64,
                                              hi & (2**64 - 1), ga.encode(), gb.encode(), ctypes.byref(st)),
                  "gp_generate_window")
    oa, ob = str(tmp_path / "oa"), str(tmp_path / "ob")
    ost = GenStats()
    oracle_lib.gpo_generate_window(order, compress, paf, oa.encode(), ob.encode(), lo >> 64, lo & (2**64 - 1),
                                   hi >> 64, hi & (2**64 - 1), ctypes.byref(ost))
    assert read(ga) == read(oa)
    assert read(gb) == read(ob)
    assert st.necklaces == ost.necklaces


def test_job_split_union(tmp_path):
    """-n 3 jobs: each job's files, sorted together, equal the single run."""
    for j in range(3):
        golay(["34", "-c", "2", "-n", "3", "-j", str(j), "gen"], tmp_path / "split")
    golay(["34", "-c", "2", "-n", "3", "sort"], tmp_path / "split")
    golay(["34", "-c", "2", "all"], tmp_path / "single")  # all: gen sort match (no uncompress step: c list of 1)
    for ab in "ab":
        assert read(str(tmp_path / "split" / "order-34" / f"34-filtered_sorted-{ab}")) == \
            read(str(tmp_path / "single" / "order-34" / f"34-filtered_sorted-{ab}"))


def test_stage_by_stage_equals_all(tmp_path):
    golay(["26", "-c", "2", "1", "gen"], tmp_path)
    golay(["26", "-c", "2", "1", "sort"], tmp_path)
    golay(["26", "-c", "2", "1", "match"], tmp_path)
    golay(["26", "-c", "2", "1", "uncompress"], tmp_path)
    _, wd = golay(["26", "-c", "2", "1", "filter"], tmp_path)
    assert read(os.path.join(wd, "26-unique")) == read(os.path.join(GOLDEN, "n26", "26-unique"))


def test_no_decomposition_returns_1(tmp_path):
    r, _ = golay(["3", "gen"], tmp_path, check=False)  # 2*3 = 6 is not a sum of two squares
    assert r.returncode == 1


def test_match_empty_input_returns_1(tmp_path):
    wd = tmp_path / "order-16"
    wd.mkdir(parents=True)
    (wd / "16-filtered_sorted-a").write_text("")
    (wd / "16-filtered_sorted-b").write_text("PSD1 0 \n")
    r, _ = golay(["16", "-c", "2", "match"], tmp_path, check=False)
    assert r.returncode == 1
    assert (wd / "16-pairs-2").exists() and (wd / "16-pairs-2").read_text() == ""


def test_uncompress_malformed_line_fails(tmp_path):
    wd = tmp_path / "order-16"
    wd.mkdir(parents=True)
    (wd / "16-pairs-2").write_text("0 0 0 2 0 0 0 2  -2 0 -2 2 2 0 2\n")  # 15 values, expected 16
    r, _ = golay(["16", "-c", "2", "1", "uncompress"], tmp_path, check=False)
    assert r.returncode != 0


def test_sort_dedups_and_orders_bytewise(tmp_path):
    lines = [b"PSD12 0 2 \n", b"PSD123 0 2 \n", b"PSD12 -2 2 \n", b"PSD12 0 2 \n", b"PSD1 2 2 \n"]
    src = tmp_path / "in"
    src.write_bytes(b"".join(lines))
    out = tmp_path / "out"
    with gp.Context(0) as ctx:
        arr = (ctypes.c_char_p * 1)(str(src).encode())
        ctx.check(ctx._lib.gp_sort(ctx.handle, ctypes.cast(arr, ctypes.c_void_p), 1, str(out).encode()), "gp_sort")
    want = b"".join(sorted(set(lines)))
    assert out.read_bytes() == want


def test_uncompress_line_ranges_split_the_work(tmp_path, golden_manifest):
    """--range_begin/--range_end/--line (parsed but unused by the
    reference): contiguous ranges, concatenated in order, give the file of
    one uncompression over all lines; --line N gives line N's pairs."""
    golay(["26", "-c", "2", "1", "gen", "sort", "match"], tmp_path)
    _, wd = golay(["26", "-c", "2", "1", "uncompress"], tmp_path)
    full = read(os.path.join(wd, "26-pairs-1"))
    assert full == read(os.path.join(GOLDEN, "n26", "26-pairs-1"))
    golay(["26", "-c", "2", "1", "uncompress", "-o", "pa", "-b", "0", "-e", "25"], tmp_path)
    golay(["26", "-c", "2", "1", "uncompress", "-o", "pb", "-b", "25"], tmp_path)
    parts = read(os.path.join(wd, "26-pa-1")) + read(os.path.join(wd, "26-pb-1"))
    assert parts == full
    # lines 1..6 one at a time add up to the range [0, 6)
    golay(["26", "-c", "2", "1", "uncompress", "-o", "p6", "-b", "0", "-e", "6"], tmp_path)
    pieces = b""
    for line in range(1, 7):
        golay(["26", "-c", "2", "1", "uncompress", "-o", "pl", "--line", str(line)], tmp_path)
        pieces += read(os.path.join(wd, "26-pl-1"))
    assert pieces == read(os.path.join(wd, "26-p6-1"))
    # a step: lines 0, 2, 4, ... and 1, 3, 5, ... together hold every pair
    golay(["26", "-c", "2", "1", "uncompress", "-o", "pe", "-s", "2"], tmp_path)
    golay(["26", "-c", "2", "1", "uncompress", "-o", "po", "-b", "1", "-s", "2"], tmp_path)
    both = read(os.path.join(wd, "26-pe-1")) + read(os.path.join(wd, "26-po-1"))
    assert sorted(both.splitlines()) == sorted(full.splitlines())


def test_uncompress_chain_equals_level_by_level(tmp_path, golden_manifest):
    """gp_uncompress_chain runs 4 -> 2 -> 1 at order 32 with the middle
    level's pairs handed over in memory; its two files equal the
    reference's (golden hashes) and one gp_uncompress_lines call per level
    reading the file back.  A line range applies to the first level only."""
    golay(["32", "-c", "4", "2", "1", "gen", "sort", "match"], tmp_path)
    wd = os.path.join(str(tmp_path), "order-32")
    p4 = os.path.join(wd, "32-pairs-4")
    meta = golden_manifest["runs"]["n32_c421"]["files"]
    big = 2 ** 63 - 1
    with gp.Context(0) as ctx:
        L = ctx._lib

        def chain(outs, first=0, end=big, step=1):
            comps = (ctypes.c_int * 3)(4, 2, 1)
            paths = (ctypes.c_char_p * 2)(*[o.encode() for o in outs])
            ctx.check(L.gp_uncompress_chain(ctx.handle, 32, ctypes.cast(comps, ctypes.c_void_p), 3, 0, p4.encode(),
                                            ctypes.cast(paths, ctypes.c_void_p), first, end, step),
                      "gp_uncompress_chain")

        def level(src, dst, c, cn, first=0, end=big, step=1):
            ctx.check(L.gp_uncompress_lines(ctx.handle, 32, c, cn, 0, src.encode(), dst.encode(), wd.encode(), b"",
                                            first, end, step), "gp_uncompress_lines")

        c2, c1 = os.path.join(wd, "chain-2"), os.path.join(wd, "chain-1")
        chain([c2, c1])
        assert hashlib.sha256(read(c2)).hexdigest() == meta["32-pairs-2"]["sha256"]
        assert hashlib.sha256(read(c1)).hexdigest() == meta["32-pairs-1"]["sha256"]
        l2, l1 = os.path.join(wd, "lvl-2"), os.path.join(wd, "lvl-1")
        level(p4, l2, 4, 2)
        level(l2, l1, 2, 1)
        assert read(l2) == read(c2) and read(l1) == read(c1)
        # every third input line from line 1
        chain([c2, c1], first=1, step=3)
        level(p4, l2, 4, 2, first=1, step=3)
        level(l2, l1, 2, 1)
        assert read(l2) == read(c2) and read(l1) == read(c1)
        assert len(read(c1)) > 0


def _filter_gpu_vs_oracle(oracle_lib, tmp_path, order, pairs_file):
    with gp.Context(0) as ctx:
        ctx.check(ctx._lib.gp_equiv_filter(ctx.handle, order, 1, str(pairs_file).encode(),
                                           str(tmp_path / "gpu").encode()), "gp_equiv_filter")
    assert oracle_lib.gpo_equiv_filter(order, 1, str(pairs_file).encode(), str(tmp_path / "orc").encode()) == 0
    got, want = read(tmp_path / "gpu"), read(tmp_path / "orc")
    assert got == want
    return got


N57 = ["57", "-c", "3", "1", "--paf", "-2"]


def test_order57_compression3_matches_reference(tmp_path, golden_manifest):
    """Order 57, paf -2, compression 3 -> 1 (Legendre-type pairs): gen, sort
    and match over the whole word space give the reference's sorted files
    (366,602 a / 3,299,242 b lines) and its 196,216-line pair file; the
    uncompression to length 57 and the equivalence filter of two 200-line
    subsets of that pair file (its first 200 lines, and 200 lines drawn with
    a fixed seed) give the reference's compression-1 pairs and unique pairs
    (the reference's outputs, produced by tests/golden/make_golden.py)."""
    rec = golden_manifest["n57"]
    _, wd = golay(N57 + ["gen", "sort", "match"], tmp_path / "full")
    for fn, meta in rec["files"].items():
        got = read(os.path.join(wd, fn))
        assert got.count(b"\n") == meta["lines"], fn
        assert hashlib.sha256(got).hexdigest() == meta["sha256"], fn
    lines = read(os.path.join(wd, "57-pairs-3")).splitlines(keepends=True)
    for name, sub in rec["subsets"].items():
        d = tmp_path / name / "order-57"
        d.mkdir(parents=True)
        (d / "57-pairs-3").write_bytes(b"".join(lines[i] for i in sub["indices"]))
        _, swd = golay(N57 + ["uncompress", "filter"], tmp_path / name)
        for fn, meta in sub["files"].items():
            got = read(os.path.join(swd, fn))
            assert got.count(b"\n") == meta["lines"], (name, fn)
            assert hashlib.sha256(got).hexdigest() == meta["sha256"], (name, fn)


def test_filter_n32_matches_oracle(oracle_lib, tmp_path, golden_manifest):
    """Equivalence filter of order-32 pairs at compression 1 (even length: the
    alternating-negation generators are in the set): the first 3000 of the
    90,320 pairs the 4 -> 2 -> 1 pipeline writes (checked against the
    reference's hash by test_gen_matches_reference_hash)."""
    _, wd = golay(golden_manifest["runs"]["n32_c421"]["argv"], tmp_path)
    lines = read(os.path.join(wd, "32-pairs-1")).splitlines(keepends=True)
    sub = tmp_path / "pairs3000"
    sub.write_bytes(b"".join(lines[:3000]))
    out = _filter_gpu_vs_oracle(oracle_lib, tmp_path, 32, sub)
    assert 0 < out.count(b"\n") < 3000


def test_filter_n57_matches_oracle(oracle_lib, tmp_path):
    """Order 57, paf -2: the pairs at compression 1 of the first 200 pairs at
    compression 3 (8208 generators per pair, several CTAs per pair)."""
    golay(["57", "-c", "3", "1", "--paf", "-2", "gen", "sort", "match"], tmp_path)
    _, wd = golay(["57", "-c", "3", "1", "--paf", "-2", "uncompress", "-e", "200"], tmp_path)
    pairs = os.path.join(wd, "57-pairs-1")
    assert read(pairs).count(b"\n") > 10
    _filter_gpu_vs_oracle(oracle_lib, tmp_path, 57, pairs)


@pytest.mark.parametrize("L", [64, 127, 128])
def test_filter_long_pairs_by_least_images(tmp_path, L):
    """Lengths whose group table the reference (and the table kernel) could
    not hold (L = 128, compression 1: 33.5 million elements of 256 entries):
    three random pairs and two images of each under known group elements
    (a shift of b with a swap, a decimation with a reversal of b, the
    alternating negation at even L) form three classes; with classes this
    small against their class sizes the reference's erase loop keeps the
    first member of each class in set order."""
    rng = np.random.default_rng(L)
    units = [u for u in range(2, L) if np.gcd(u, L) == 1]

    def images(a, b):
        i = np.arange(L)
        out = [(np.roll(b, -5), a)]                           # shift b by 5, then swap
        u = units[len(units) // 2]
        a2, b2 = a[(u * i) % L], b[(u * i) % L]               # decimate both by u
        out.append((a2, b2[::-1].copy()))                     # reverse b
        if L % 2 == 0:
            sg = np.where(i % 2 == 1, -1, 1)
            out.append((a * sg, b * sg))                      # alternating negation
        return out

    pairs = []
    classes = []
    for _ in range(3):
        a = rng.choice([-1, 1], L).astype(np.int8)
        b = rng.choice([-1, 1], L).astype(np.int8)
        cls = [(a, b)] + images(a, b)
        keys = [tuple(int(v) for v in np.concatenate([x, y])) for x, y in cls]
        classes.append(sorted(set(keys)))
        pairs += keys
    src = tmp_path / "pairs"
    src.write_text("".join(" ".join(map(str, p[:L])) + "  " + " ".join(map(str, p[L:])) + "\n" for p in pairs))
    out = tmp_path / "unique"
    with gp.Context(0) as ctx:
        ctx.check(ctx._lib.gp_equiv_filter(ctx.handle, L, 1, str(src).encode(), str(out).encode()), "gp_equiv_filter")
    want = sorted(c[0] for c in classes)
    got = [tuple(int(v) for v in line.split()) for line in read(out).decode().splitlines()]
    assert got == want


def _lines(path):
    return read(path).count(b"\n")


def test_spectral_prune_keeps_reference_pairs_n16(tmp_path, golden_manifest):
    """Length 8 (even): gen --spectral-prune writes fewer candidates, and the
    sorted-match pairs are still the reference's."""
    files = golden_manifest["runs"]["n16"]["files"]
    _, wd = golay(["16", "-c", "2", "gen", "--spectral-prune", "sort", "match"], tmp_path)
    assert hashlib.sha256(read(os.path.join(wd, "16-pairs-2"))).hexdigest() == files["16-pairs-2"]["sha256"]
    kept = _lines(os.path.join(wd, "16-filtered-a#0")) + _lines(os.path.join(wd, "16-filtered-b#0"))
    assert kept < files["16-filtered-a#0"]["lines"] + files["16-filtered-b#0"]["lines"]


def test_spectral_prune_keeps_reference_pairs_n32(tmp_path, golden_manifest):
    """Order 32 at compression 4 (length 8), uncompressed 4 -> 2 -> 1: every
    pair file equals the reference's."""
    rec = golden_manifest["runs"]["n32_c421"]
    argv = list(rec["argv"])
    argv.insert(argv.index("gen") + 1, "--spectral-prune")
    _, wd = golay(argv, tmp_path)
    for fn in ("32-pairs-4", "32-pairs-2", "32-pairs-1"):
        assert hashlib.sha256(read(os.path.join(wd, fn))).hexdigest() == rec["files"][fn]["sha256"], fn


@pytest.mark.parametrize("order,compress,paf", [(36, 2, 0), (21, 1, -2)])
def test_spectral_prune_same_pairs(tmp_path, order, compress, paf):
    """Lengths 18 (both the L/2 and the L/3 test apply) and 21 (the L/3 test):
    the same pair file with and without pruning, from no more candidates."""
    args = [str(order), "-c", str(compress), "--paf", str(paf)]
    _, w0 = golay(args + ["gen", "sort", "match"], tmp_path / "plain")
    _, w1 = golay(args + ["gen", "--spectral-prune", "sort", "match"], tmp_path / "pruned")
    pairs = f"{order}-pairs-{compress}"
    assert read(os.path.join(w1, pairs)) == read(os.path.join(w0, pairs))
    n0 = _lines(os.path.join(w0, f"{order}-filtered_sorted-a")) + _lines(os.path.join(w0, f"{order}-filtered_sorted-b"))
    n1 = _lines(os.path.join(w1, f"{order}-filtered_sorted-a")) + _lines(os.path.join(w1, f"{order}-filtered_sorted-b"))
    assert n1 < n0


def test_spectral_identity_at_third_bin_order57(tmp_path):
    """p_A(L/3) + p_B(L/3) = 2n - paf on the order-57 pairs at compression 1
    (length 57): the identity the L/3 test rests on, on real pairs."""
    golay(["57", "-c", "3", "1", "--paf", "-2", "gen", "sort", "match"], tmp_path)
    _, wd = golay(["57", "-c", "3", "1", "--paf", "-2", "uncompress", "-e", "200"], tmp_path)
    lines = read(os.path.join(wd, "57-pairs-1")).decode().splitlines()
    assert lines
    for line in lines:
        v = [int(x) for x in line.split()]
        pa = np.abs(np.fft.fft(np.array(v[:57]))) ** 2
        pb = np.abs(np.fft.fft(np.array(v[57:]))) ** 2
        assert abs(pa[19] + pb[19] - (2 * 57 + 2)) < 1e-6
        assert abs(pa[19] - round(pa[19])) < 1e-6


def test_every_emitted_pair_is_complementary_order57(tmp_path):
    """Property over all 196,216 pairs match writes at order 57 (paf -2,
    compression 3): PAF_a(s) + PAF_b(s) = paf * c for s = 1 .. L/2, the
    reference's check_if_pair (src/utils/golay.cpp:27-44)."""
    _, wd = golay(["57", "-c", "3", "--paf", "-2", "gen", "sort", "match"], tmp_path)
    arr = np.array(read(os.path.join(wd, "57-pairs-3")).split(), dtype=np.int64).reshape(-1, 38)
    assert len(arr) == 196216
    a, b = arr[:, :19], arr[:, 19:]
    for s in range(1, 10):
        paf = (a * np.roll(a, -s, axis=1)).sum(axis=1) + (b * np.roll(b, -s, axis=1)).sum(axis=1)
        assert (paf == -2 * 3).all(), s


def test_sort_of_a_missing_file_fails(tmp_path):
    """Injected failure: the sort stage with an input file that does not
    exist reports the error (the reference's GNU_sort returns 1,
    src/core/sort/sort.cpp:18-21)."""
    r, _ = golay(["26", "-c", "2", "sort"], tmp_path, check=False)
    assert r.returncode != 0
    assert "sort" in (r.stderr + r.stdout).lower()
