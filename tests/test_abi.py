"""The C ABI library: every entry point include/*.h declares is exported, the
structs have the reference's sizes, and without a GPU the backend refuses
clearly instead of misbehaving (tests/test_gpu_kernels.cpp:355-370)."""

import ctypes as C
import pathlib
import re

import pytest

from conftest import have_gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared(header):
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(gtc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(gtc):
    names = declared(ROOT / "include" / "gtc.h")
    assert len(names) >= 15
    missing = [s for s in names if not hasattr(gtc.lib, s)]
    assert missing == []


def test_struct_sizes(gtc):
    assert C.sizeof(gtc.KernelParams) == 32      # GTParams, metal_backend.mm:22
    assert gtc.NODE_DTYPE.itemsize == 144
    assert C.sizeof(gtc.GravityParams) == 56


def test_status_names(gtc):
    assert gtc.lib.gtc_status_name(gtc.GTC_INVALID_ARGUMENT) == b"invalid argument"


@pytest.mark.skipif(have_gpu(), reason="checks the refusal without a device")
def test_refuses_without_device(gtc):
    with pytest.raises(gtc.GtcError) as e:
        gtc.Context(0)
    assert e.value.status == gtc.GTC_NO_DEVICE
    assert "no GPU" in str(e.value)
