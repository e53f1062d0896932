"""Binary survivor files, host side: an independent Python writer of the
format turns the reference's own candidate files (tests/golden) into binary
survivor files, and gp_export_text must give back the reference's bytes.
Runs on the CPU (the exporter needs no GPU)."""
import os
import struct

import numpy as np
import pytest

import golaypair_gb300 as gp
from conftest import GOLDEN, read

MAGIC = b"GPSURV01"


def alphabet(c):
    # src/utils/golay.cpp:60-75
    if c % 2 == 0:
        return list(range(-c, c + 1, 2))
    return list(range(-c, 0, 2)) + list(range(1, c + 1, 2))


def bits_for(k):
    b = 1
    while (1 << b) < k:
        b += 1
    return b


def encode(text, order, compress, paf, role):
    """Binary survivor file of a candidate text file: the signature values
    are recomputed in FP64 from each line's entries (the line only holds
    them concatenated) and checked against the line."""
    L = order // compress
    alpha = alphabet(compress)
    k, b = len(alpha), bits_for(len(alpha))
    bound = 2 * order - paf
    recs, sig_max = [], 0
    for line in text.decode().splitlines():
        head, *entries = line.split(" ")
        seq = [int(x) for x in entries if x != ""]
        assert len(seq) == L
        psd = np.abs(np.fft.fft(np.array(seq, dtype=np.float64))) ** 2
        vals = np.rint(psd[1:]).astype(np.int64)
        if role == 1:
            vals = bound - vals
        assert head == "PSD" + "".join(str(v) for v in vals), line
        word = 0
        for x in seq:
            word = (word << b) | alpha.index(x)
        recs.append((word, [int(v) for v in vals]))
        sig_max = max([sig_max] + [int(v) for v in vals])
    sig_bytes = 1 if sig_max <= 255 else 2
    word_bytes = (b * L + 7) // 8
    hdr = MAGIC + struct.pack("<I9iQ", 1, order, compress, paf, L, k, b, role, sig_bytes, word_bytes, len(recs))
    hdr += struct.pack("<16b", *(alpha + [0] * (16 - k))) + bytes(8)
    assert len(hdr) == 80
    body = bytearray()
    for word, vals in recs:
        body += word.to_bytes(word_bytes, "little")
        for v in vals:
            body += v.to_bytes(sig_bytes, "little")
    return hdr + bytes(body)


CASES = [("n16", 16, 2, 0), ("n26", 26, 2, 0)]


@pytest.mark.parametrize("name,order,compress,paf", CASES)
@pytest.mark.parametrize("ab,role", [("a", 0), ("b", 1)])
def test_export_gives_reference_text(tmp_path, name, order, compress, paf, ab, role):
    text = read(os.path.join(GOLDEN, name, f"{order}-filtered-{ab}_0"))
    binf = tmp_path / "surv.bin"
    binf.write_bytes(encode(text, order, compress, paf, role))
    assert binf.stat().st_size < len(text)
    out = tmp_path / "out.txt"
    gp.export_text(binf, out)
    assert out.read_bytes() == text


def test_export_of_an_empty_file(tmp_path):
    binf = tmp_path / "e.bin"
    binf.write_bytes(encode(b"", 26, 2, 0, 0))
    gp.export_text(binf, tmp_path / "e.txt")
    assert (tmp_path / "e.txt").read_bytes() == b""


def test_export_rejects_malformed_files(tmp_path):
    good = encode(read(os.path.join(GOLDEN, "n26", "26-filtered-a_0")), 26, 2, 0, 0)
    cases = {
        "text": read(os.path.join(GOLDEN, "n26", "26-filtered-a_0")),
        "truncated": good[:-1],
        "short_header": good[:40],
        "bad_version": good[:8] + struct.pack("<I", 2) + good[12:],
        # alphabet of 3 letters in 2-bit digits: digit 3 does not exist
        "bad_digit": good[:80] + bytes([0xFF]) + good[81:],
    }
    for name, data in cases.items():
        p = tmp_path / name
        p.write_bytes(data)
        with pytest.raises(gp.GPError):
            gp.export_text(p, tmp_path / (name + ".txt"))


def test_cli_export_runs_without_a_gpu(tmp_path):
    """`golay 26 -c 2 export` turns this job's binary files into the
    reference's text in place, on the host."""
    import subprocess
    wd = tmp_path / "order-26"
    wd.mkdir()
    for ab, role in (("a", 0), ("b", 1)):
        text = read(os.path.join(GOLDEN, "n26", f"26-filtered-{ab}_0"))
        (wd / f"26-filtered-{ab}#0").write_bytes(encode(text, 26, 2, 0, role))
    r = subprocess.run([gp.CLI_PATH, "26", "-c", "2", "--dir", str(tmp_path), "export"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    for ab in "ab":
        assert (wd / f"26-filtered-{ab}#0").read_bytes() == read(os.path.join(GOLDEN, "n26", f"26-filtered-{ab}_0"))


@pytest.mark.parametrize("name,order,fn,L", [("n16", 16, "16-pairs-2", 8), ("n16", 16, "16-pairs-1", 16),
                                             ("n26", 26, "26-pairs-1", 26)])
def test_spectral_identity_on_reference_pairs(name, order, fn, L):
    """The identity spectral pruning rests on, on the reference's own pairs:
    p_A(k) + p_B(k) = 2n - paf for every k != 0, in particular at k = L/2
    where both are squares of integers (the alternating sums)."""
    bound = 2 * order
    lines = read(os.path.join(GOLDEN, name, fn)).decode().splitlines()
    assert lines
    sign = np.array([(-1) ** j for j in range(L)])
    for line in lines:
        v = [int(x) for x in line.split()]
        a, b = np.array(v[:L]), np.array(v[L:])
        pa = np.abs(np.fft.fft(a)) ** 2
        pb = np.abs(np.fft.fft(b)) ** 2
        assert np.allclose(pa[1:] + pb[1:], bound, atol=1e-6)
        sa, sb = int(a @ sign), int(b @ sign)
        assert sa * sa + sb * sb == bound


def test_export_two_byte_signatures(tmp_path):
    """Order 140 at compression 4 (length 35, five letters in 3-bit digits):
    the bound 280 needs 2-byte signature fields.  Records with arbitrary
    values; the expected lines are written here from the line format."""
    order, compress, paf, role = 140, 4, 0, 1
    L, alpha, b = 35, [-4, -2, 0, 2, 4], 3
    rng = np.random.default_rng(11)
    recs = [(rng.integers(0, 5, size=L), rng.integers(0, 281, size=L - 1)) for _ in range(500)]
    word_bytes = (b * L + 7) // 8
    hdr = MAGIC + struct.pack("<I9iQ", 1, order, compress, paf, L, len(alpha), b, role, 2, word_bytes, len(recs))
    hdr += struct.pack("<16b", *(alpha + [0] * 11)) + bytes(8)
    body, want = bytearray(), []
    for digits, sig in recs:
        word = 0
        for d in digits:
            word = (word << b) | int(d)
        body += word.to_bytes(word_bytes, "little")
        for v in sig:
            body += int(v).to_bytes(2, "little")
        want.append("PSD" + "".join(str(int(v)) for v in sig) + " " + "".join(f"{alpha[d]} " for d in digits) + "\n")
    (tmp_path / "s.bin").write_bytes(hdr + bytes(body))
    gp.export_text(tmp_path / "s.bin", tmp_path / "s.txt")
    assert (tmp_path / "s.txt").read_text() == "".join(want)
