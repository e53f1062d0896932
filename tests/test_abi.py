"""The C-ABI library loads on CPU and exports every symbol the public header
declares (no compute call: there is no GPU here)."""
import ctypes
import os
import subprocess

import pytest

import golaypair_gb300 as gp


@pytest.fixture(scope="module")
def built():
    gp.build()
    return gp.LIB_PATH


def test_library_exports_header_symbols(built):
    lib = ctypes.CDLL(built)
    names = gp.header_symbols()
    assert "gp_psd_filter" in names and "gp_ctx_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_context_fails_loudly_without_gpu(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(gp.GPError):
        gp.Context(0)


def test_cli_built(built):
    if not os.path.exists(gp.CLI_PATH):
        pytest.skip("CLI not built yet")
    r = subprocess.run([gp.CLI_PATH, "--help"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert "order" in r.stdout
