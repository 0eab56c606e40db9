"""The evaluators' rsqrt (csrc/common.cuh, rsqrt_normal: the SFU instruction
without rsqrtf's subnormal-input handling) returns rsqrtf's value bit for
bit on every positive normal float -- every r^2 the softened evaluators
take -- so the forces do not change with it."""

import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.mark.gpu
def test_rsqrt_normal_equals_rsqrtf_on_every_normal_float(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "rsqrt_normal_check"
    subprocess.run([nvcc, "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
                    str(ROOT / "tests" / "cuda" / "rsqrt_normal_check.cu"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    fields = out.split()
    assert fields[fields.index("checked") + 1] == str(0x7F800000 - 0x00800000)
    assert fields[fields.index("mismatches") + 1] == "0", out
