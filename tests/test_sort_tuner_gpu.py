"""gp_sort's radix-width tuner: on inputs large enough to time it picks 4-
or 8-bit passes per key width, caches the choice in the context, and the
output stays `sort | uniq` in byte order."""
import ctypes

import numpy as np
import pytest

import golaypair_gb300 as gp

pytestmark = pytest.mark.gpu


def candidate_lines(rng, n, L):
    sig = rng.integers(0, 60, size=(n, L - 1))
    vals = rng.choice(np.array([-2, 0, 2]), size=(n, L))
    out = []
    for s, v in zip(sig, vals):
        out.append(("PSD" + "".join(map(str, s)) + " " + "".join(f"{x} " for x in v) + "\n").encode())
    return out


@pytest.mark.parametrize("n,L", [(60_000, 17), (40_000, 34)])
def test_sort_tuner_matches_bytewise_sort(tmp_path, n, L):
    rng = np.random.default_rng(n + L)
    lines = candidate_lines(rng, n, L)
    lines += lines[: n // 5]  # duplicates
    rng.shuffle(lines)
    src = tmp_path / "in"
    src.write_bytes(b"".join(lines))
    want = b"".join(sorted(set(lines)))
    with gp.Context(0) as ctx:
        for rep in range(2):
            out = tmp_path / f"out{rep}"
            paths = (ctypes.c_char_p * 1)(str(src).encode())
            ctx.check(ctx._lib.gp_sort(ctx.handle, ctypes.cast(paths, ctypes.c_void_p), 1, str(out).encode()),
                      "gp_sort")
            assert out.read_bytes() == want
        tuned = {k: v for k, v in ctx.tuned_settings().items() if k.startswith("sort:W")}
        assert len(tuned) == 1
        assert list(tuned.values())[0][0] in (4, 8)
