"""The C-ABI library builds, loads and exports every function that
include/gbrt.h declares; the Python mirrors of the structs have the sizes
the header's static_asserts pin.  No GPU work runs here."""
import os
import re

import ctypes as C

import pytest

from rustracer_gb300 import build, gbrt, types as T

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbrt.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(gbrt_\w+)\s*\(", src, flags=re.M)))


def test_header_parses():
    fns = declared_functions()
    assert "gbrt_render" in fns and "gbrt_tlas_build" in fns and len(fns) >= 25


def test_library_exports_every_declared_symbol():
    build.build()
    L = gbrt.load()
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing
    assert set(declared_functions()) == set(gbrt.SIGNATURES), "bindings out of sync with the header"


def test_version_string():
    assert gbrt.load().gbrt_version().decode().startswith("gbrt")


def test_struct_sizes():
    assert T.VERTEX.itemsize == 128 and T.MATERIAL.itemsize == 256 and T.UBO.itemsize == 324
    assert T.LIGHT.itemsize == 48 and T.INSTANCE.itemsize == 64 and T.PRIMINFO.itemsize == 16
    assert T.JOB_INFO.itemsize == 128 and C.sizeof(gbrt.JobDesc) == 64
    assert C.sizeof(gbrt.NrcConfig) == 56 and C.sizeof(gbrt.NrcRenderOpts) == 20


def test_no_device_is_an_error_not_a_crash():
    """Without a GPU, context creation fails with GBRT_E_NO_DEVICE (or
    GBRT_E_CUDA) and a message; it never falls back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gbrt.GbrtError) as e:
        gbrt.Context(0)
    assert e.value.code in (gbrt.E_NO_DEVICE, gbrt.E_CUDA)
