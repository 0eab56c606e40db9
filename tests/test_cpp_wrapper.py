"""The C++ wrapper (galactic-tides_gb300/host/gtc.hpp): a C++ program in the
reference's test style, built with g++ against libgtc.so and the oracle, run
on the GPU; and, where the reference's headers are present, a compile check of
the drop-in backend (galactic-tides_gb300/host/gravity_backends_cuda.cpp)
against them. The reference's location comes from the oracle/_ref build,
which records it in oracle/_ref/REFERENCE."""

import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
PKG = ROOT / "galactic-tides_gb300"

def reference_include():
    """include/ of the reference tree oracle/_ref was built from, if any."""
    rec = ROOT / "oracle" / "_ref" / "REFERENCE"
    if not rec.exists():
        return None
    inc = pathlib.Path(rec.read_text().strip()) / "include"
    return inc if (inc / "galactic_tides" / "integrator.h").exists() else None


def compile_cpp(src, out, extra=()):
    cmd = ["g++", "-std=c++17", "-O2", str(src), "-o", str(out), f"-I{ROOT / 'include'}",
           f"-I{PKG / 'host'}", f"-L{PKG}", "-lgtc", f"-Wl,-rpath,{PKG}", *extra]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


@pytest.mark.gpu
def test_cpp_wrapper_program(tmp_path):
    exe = tmp_path / "test_host_wrapper"
    compile_cpp(ROOT / "tests" / "cpp" / "test_host_wrapper.cpp", exe,
                [f"-L{ROOT / 'oracle'}", "-loracle", f"-Wl,-rpath,{ROOT / 'oracle'}"])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout


@pytest.mark.skipif(reference_include() is None, reason="needs the reference's headers")
def test_integration_backend_compiles_against_reference(tmp_path):
    """CudaGroupGravity / CudaDirectGravity (the file INTEGRATION.md shows),
    compiled against the reference's own ForceModel and Particles."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = PKG / "host" / "gravity_backends_cuda.cpp"
    cmd = ["g++", "-std=c++17", "-c", str(src), "-o", str(tmp_path / "x.o"),
           f"-I{reference_include()}", f"-I{ROOT / 'include'}", f"-I{PKG / 'host'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
