"""The ABI from plain C: tests/c_abi/abi_client.c is compiled with gcc against
include/kbwg.h and linked to kbw_gb300/libkbwg.so, as a non-Python host (the
Rust shim, a C plugin) would use it.  Without a GPU it must link and fail
cleanly (status codes, no crash); on a GPU it runs Bell/GHZ states through
the trait-style calls, readout, error paths and a batch entry."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_abi", "abi_client.c")
LIBDIR = os.path.join(ROOT, "kbw_gb300")


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    if not os.path.exists(os.path.join(LIBDIR, "libkbwg.so")):
        import __graft_entry__
        __graft_entry__.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("c_abi") / "abi_client")
    cmd = [cc, "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", LIBDIR, "-lkbwg", "-Wl,-rpath," + LIBDIR, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_client_links_and_fails_cleanly_without_gpu(client, cuda_available):
    if cuda_available:
        pytest.skip("GPU present: the GPU test runs the client")
    r = subprocess.run([client, "--no-gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_c_client_on_gpu(client):
    r = subprocess.run([client], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok (0 failures)")
