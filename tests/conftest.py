"""Shared fixtures: builds the CPU oracle (the checker) and, for GPU tests,
loads the product library through its C ABI."""
import ctypes
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU runs")


@pytest.fixture(scope="session")
def oracle_bin():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True, stdout=subprocess.DEVNULL)
    return os.path.join(ORACLE_BUILD, "golay_oracle")


@pytest.fixture(scope="session")
def oracle_lib(oracle_bin):
    return load_oracle()


def load_oracle():
    lib = ctypes.CDLL(os.path.join(ORACLE_BUILD, "libgolay_oracle.so"))
    i32, i64, u64 = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64
    P = ctypes.c_void_p
    lib.gpo_alphabet.argtypes = [i32, P]
    lib.gpo_decomps.argtypes = [i32, P, P, i32]
    lib.gpo_psd.argtypes = [P, i32, P]
    lib.gpo_is_canonical.argtypes = [P, i32, i32]
    lib.gpo_orderly_generators.argtypes = [i32, i32, P, i32]
    lib.gpo_check_if_pair.argtypes = [P, P, i32, i32, i32]
    lib.gpo_generate.argtypes = [i32, i32, i32, ctypes.c_char_p, ctypes.c_char_p, i32, i32, P]
    lib.gpo_generate_window.argtypes = [i32, i32, i32, ctypes.c_char_p, ctypes.c_char_p, u64, u64, u64, u64, P]
    lib.gpo_sort.argtypes = [P, i32, ctypes.c_char_p]
    lib.gpo_match.argtypes = [i32, i32, i32, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i32, P]
    lib.gpo_uncompress.argtypes = [i32, i32, i32, i32, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                   ctypes.c_char_p]
    lib.gpo_uncompress_one.argtypes = [P, i32, i32, i32, i32, i32, ctypes.c_char_p, P, P]
    lib.gpo_equiv_filter.argtypes = [i32, i32, ctypes.c_char_p, ctypes.c_char_p]
    lib.gpo_pair_generator_count.argtypes = [i32, i32]
    lib.gpo_pair_generator_count.restype = i64
    lib.gpo_necklace_count.argtypes = [i32, i32]
    lib.gpo_necklace_count.restype = i64
    lib.gpo_psd_filter_batch.argtypes = [P, i64, i32, i32, i32, P, i32]
    lib.gpo_psd_filter_batch.restype = i64
    lib.gpo_psd_max_batch.argtypes = [P, i64, i32, P, i32]
    return lib


class GenStats(ctypes.Structure):
    _fields_ = [("necklaces", ctypes.c_int64), ("psd_evals", ctypes.c_int64), ("psd_pass", ctypes.c_int64),
                ("written_a", ctypes.c_int64), ("written_b", ctypes.c_int64)]


@pytest.fixture(scope="session")
def golden_manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def read(path):
    with open(path, "rb") as f:
        return f.read()
