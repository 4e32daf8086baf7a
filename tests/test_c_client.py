"""The C ABI from a C program (tests/c_client.c), compiled with gcc against
include/goldilocks_gpu.h and the in-tree library, as a foreign-function
binding of the reference's Ntt slot would use it: host-side calls on the CPU,
transforms of a host buffer on the GPU."""
import os
import subprocess

import pytest

from conftest import ROOT

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def client(gl, tmp_path_factory):
    from goldilocks_gb300 import build
    lib = build.LIB
    exe = tmp_path_factory.mktemp("c_client") / "c_client"
    subprocess.run(["gcc", "-std=c11", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c_client.c"), lib, "-Wl,-rpath," + os.path.dirname(lib),
                    "-o", str(exe)], check=True)
    return str(exe)


def test_c_client_host_calls(client):
    out = subprocess.run([client, "host"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "ok"


@pytest.mark.gpu
def test_c_client_transforms(client):
    out = subprocess.run([client, "gpu"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "ok"
