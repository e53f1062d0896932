"""Pins the CPU oracle against the reference's own outputs (golden fixtures
generated by tests/golden/make_golden.py from the reference sources)."""
import ctypes
import hashlib
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, GenStats, read

ENV = dict(os.environ, LC_ALL="C")


def run_oracle(oracle_bin, tmp_path, argv):
    d = str(tmp_path / "res")
    subprocess.run([oracle_bin] + argv[:-1] + ["--dir", d, argv[-1]], check=True, env=ENV,
                   stdout=subprocess.DEVNULL)
    return os.path.join(d, f"order-{argv[0]}")


@pytest.mark.parametrize("name", ["n16", "n26", "n21_c31", "n27_c31"])
def test_oracle_full_pipeline_matches_reference(oracle_bin, tmp_path, golden_manifest, name):
    rec = golden_manifest["runs"][name]
    wd = run_oracle(oracle_bin, tmp_path, rec["argv"])
    for fn, meta in rec["files"].items():
        got = read(os.path.join(wd, fn))
        assert got == read(os.path.join(GOLDEN, name, fn.replace("#", "_"))), fn
        assert got.count(b"\n") == meta["lines"]


@pytest.mark.parametrize("name", ["n34", "n57_shard7of1000", "n33_c31"])
def test_oracle_generation_matches_reference_hash(oracle_bin, tmp_path, golden_manifest, name):
    rec = golden_manifest["runs"][name]
    wd = run_oracle(oracle_bin, tmp_path, rec["argv"])
    for fn, meta in rec["files"].items():
        got = read(os.path.join(wd, fn))
        assert hashlib.sha256(got).hexdigest() == meta["sha256"], fn
        assert got.count(b"\n") == meta["lines"]


def _units(L):
    return [u for u in range(1, L) if math.gcd(u, L) == 1] if L > 1 else [1]


@pytest.mark.parametrize("L", list(range(1, 41)) + [45, 57])
def test_orderly_generators_are_affine_and_dihedral(oracle_lib, L):
    """constructGenerators(0, L) is the affine group i -> u*i + t (u a unit),
    constructGenerators(1, L) the dihedral group i -> +-i + t; the GPU
    canonical check relies on this characterisation."""
    for flag in (0, 1):
        n = oracle_lib.gpo_orderly_generators(L, flag, None, 0)
        buf = (ctypes.c_int * (n * L))()
        oracle_lib.gpo_orderly_generators(L, flag, buf, n)
        got = {tuple(buf[i * L:(i + 1) * L]) for i in range(n)}
        mults = _units(L) if flag == 0 else [1, L - 1 if L > 1 else 1]
        want = {tuple((u * i + t) % L for i in range(L)) for u in mults for t in range(L)}
        assert got == want


def test_necklace_counts(oracle_lib):
    assert oracle_lib.gpo_necklace_count(8, 3) == 834
    assert oracle_lib.gpo_necklace_count(13, 3) == 122643
    assert oracle_lib.gpo_necklace_count(17, 3) == 7596483


@pytest.mark.parametrize("order,compress,paf,nwin", [(16, 2, 0, 7), (26, 2, 0, 5), (34, 2, 0, 3)])
def test_window_union_equals_full_enumeration(oracle_lib, tmp_path, order, compress, paf, nwin):
    """Rank windows that partition the word space reproduce the full run."""
    L = order // compress
    k = len([v for v in range(-compress, compress + 1, 2) if compress % 2 == 0 or v % 2 != 0])
    total = k ** L
    full_a, full_b = str(tmp_path / "fa"), str(tmp_path / "fb")
    st = GenStats()
    assert oracle_lib.gpo_generate(order, compress, paf, full_a.encode(), full_b.encode(), 0, 1,
                                   ctypes.byref(st)) == 0
    bounds = [0] + sorted(np.random.default_rng(1).integers(1, total, nwin - 1).tolist()) + [total]
    cat_a, cat_b = b"", b""
    for w in range(nwin):
        lo, hi = bounds[w], bounds[w + 1]
        pa, pb = str(tmp_path / f"a{w}"), str(tmp_path / f"b{w}")
        oracle_lib.gpo_generate_window(order, compress, paf, pa.encode(), pb.encode(), lo >> 64,
                                       lo & (2**64 - 1), hi >> 64, hi & (2**64 - 1), None)
        cat_a += read(pa)
        cat_b += read(pb)
    assert cat_a == read(full_a)
    assert cat_b == read(full_b)


def test_pair_generator_sizes(oracle_lib):
    # printed by the reference's generateExhaust for n=16, c=1 (65536 items)
    assert oracle_lib.gpo_pair_generator_count(16, 1) == 65536


def test_psd_batch_matches_scalar(oracle_lib):
    rng = np.random.default_rng(0)
    L, order = 13, 26
    seqs = rng.choice(np.array([-2, 0, 2], dtype=np.int8), size=(500, L))
    ver = np.zeros(500, dtype=np.uint8)
    n = oracle_lib.gpo_psd_filter_batch(seqs.ctypes.data, 500, L, order, 0, ver.ctypes.data, 3)
    psd = (ctypes.c_double * L)()
    for i in range(500):
        s = (ctypes.c_int * L)(*seqs[i].tolist())
        oracle_lib.gpo_psd(s, L, psd)
        ok = all(psd[k] <= 2 * order + 0.001 for k in range(1, L // 2 + 1))
        assert ver[i] == ok
    assert n == ver.sum()


@pytest.mark.parametrize("compress", [1, 2])
def test_pair_generator_set_matches_oracle_closure(oracle_lib, compress):
    """gp_equiv_filter builds the generator group from a generating subset
    of the reference's operations; its size must equal the oracle's closure
    under all of them (the subset's closure is contained in the full one, so
    equal sizes mean equal sets)."""
    import golaypair_gb300 as gp
    lib = gp.lib()
    for L in range(2, 23):
        assert lib.gp_debug_pair_generator_count(L, compress) == oracle_lib.gpo_pair_generator_count(L, compress), L
    # 4 phi(L) L^2 (x 8 at compression 1, even L) for L >= 3; too large a table is refused
    assert lib.gp_debug_pair_generator_count(57, compress) == 4 * 36 * 57 * 57
    assert lib.gp_debug_pair_generator_count(128, 1) == -1


@pytest.mark.parametrize("compress", [1, 2, 3])
def test_pair_group_affine_description_equals_closure(compress):
    """For L >= 3 gp_equiv_filter finds classes by least images over an
    affine description of the pair group (swap, multiplier +-u, a shift per
    half, the alternating signs at compression 1 and even L); that
    description must give exactly the closure's elements."""
    import golaypair_gb300 as gp
    lib = gp.lib()
    for L in list(range(3, 27)) + [32, 39]:
        assert lib.gp_debug_pair_group_check(L, compress) == 1, (L, compress)
    assert lib.gp_debug_pair_group_check(2, compress) == -1


# Known answers recorded in the reference's notes (NOTES.md:455,459 and :436)
NOTES_ORDER26_A = [-1, -1, -1, -1, 1, 1, -1, -1, 1, 1, 1, -1, 1, -1, 1, -1, 1, 1, -1, 1, 1, -1, 1, 1, 1, 1]
NOTES_ORDER26_A_C2 = [-2, 0, -2, 0, 2, 0, 0, 0, 0, 2, 2, 0, 2]
NOTES_ORDER72_C6 = ([-6, 0, 0, 0, 0, 0, 6, 0, 0, 0, 0, 0], [0, 0, 0, 0, 0, 6, 0, 0, 0, 0, 0, 6])


def test_notes_order26_candidate_has_a_representative():
    """The order-26 A candidate of the notes compresses (entry j + entry j+13)
    to the recorded 2-compressed form, and the reference's order-26 A file
    holds a member of that form's class (shifts, decimations by units,
    reversal: the A-side equivalences)."""
    a, L = NOTES_ORDER26_A, 13
    assert [a[j] + a[j + L] for j in range(L)] == NOTES_ORDER26_A_C2
    x = NOTES_ORDER26_A_C2
    orbit = set()
    for u in (u for u in range(1, L) if math.gcd(u, L) == 1):
        for s in range(L):
            y = tuple(x[(s + u * i) % L] for i in range(L))
            orbit.add(y)
            orbit.add(y[::-1])
    lines = read(os.path.join(GOLDEN, "n26", "26-filtered-a_0")).decode().splitlines()
    seqs = {tuple(int(v) for v in ln.split()[1:]) for ln in lines}
    assert orbit & seqs


def test_notes_order72_compression6_candidate_is_a_pair(oracle_lib):
    """The order-72, compression-6 candidate the notes record (found by a
    generation run and matching a published compression) is a complementary
    compressed pair for the reference's check_if_pair as it stands (the notes
    describe an earlier version rejecting it): every PAF sum is 0 and every
    PSD sum is 2n = 144."""
    a, b = (np.array(v, dtype=np.int32) for v in NOTES_ORDER72_C6)
    assert oracle_lib.gpo_check_if_pair(a.ctypes.data, b.ctypes.data, 12, 0, 6) == 1
    assert [int((a * np.roll(a, -s)).sum() + (b * np.roll(b, -s)).sum()) for s in range(1, 7)] == [0] * 6
    psd = np.abs(np.fft.fft(a)) ** 2 + np.abs(np.fft.fft(b)) ** 2
    assert np.allclose(psd[1:], 144)


@pytest.mark.parametrize("L,compress", [(26, 1), (30, 1), (27, 2)])
def test_keyed_group_matches_oracle_closure(oracle_lib, L, compress):
    """The library builds the pair group by 64-bit keys of its elements; the
    oracle closes the reference's operations comparing whole items.  Sizes at
    lengths past the range above, with and without the alternating
    negation."""
    import golaypair_gb300 as gp
    assert gp.lib().gp_debug_pair_generator_count(L, compress) == oracle_lib.gpo_pair_generator_count(L, compress)
