"""Named search workloads shared by the benchmark and the tests.

The uneven batch: Golay orders 34, 50, 58, 68 at compression 2 (lengths 17,
25, 29, 34 over {-2, 0, 2}) and order 90 at compression 5 (length 18 over
{-5, -3, -1, 1, 3, 5}).  A word space no larger than the window is
enumerated whole; a larger one is searched over a 2^32-word window of
lexicographic ranks.  The window starts at a seed-drawn necklace: the least
rotation of a word drawn uniformly with numpy's default generator seeded
by order * 1000 + compression.  (A window drawn uniformly over all ranks
almost always lies where the first entry is not the smallest letter, and
such words are not necklaces: the window would hold none.)
"""
import numpy as np

BATCH_ORDERS = ((34, 2), (50, 2), (58, 2), (68, 2), (90, 5))
WINDOW_WORDS = 1 << 32


def alphabet_size(compress):
    """|alphabet|: {-c, -c+2, ..., c} has c + 1 values for even and odd c."""
    return compress + 1


def word_rank(digits, k):
    r = 0
    for d in digits:
        r = r * k + int(d)
    return r


def necklace_anchor(order, compress, seed):
    """Rank of the least rotation of a seeded uniform word."""
    L, k = order // compress, alphabet_size(compress)
    d = [int(x) for x in np.random.default_rng(seed).integers(0, k, L)]
    return word_rank(min(tuple(d[i:] + d[:i]) for i in range(L)), k)


def batch_windows(size=WINDOW_WORDS, orders=BATCH_ORDERS, paf=0):
    """(order, compress, paf, begin, end) of every job of the uneven batch."""
    out = []
    for order, comp in orders:
        space = alphabet_size(comp) ** (order // comp)
        if space <= size:
            out.append((order, comp, paf, 0, space))
        else:
            lo = necklace_anchor(order, comp, order * 1000 + comp)
            out.append((order, comp, paf, lo, min(lo + size, space)))
    return out
