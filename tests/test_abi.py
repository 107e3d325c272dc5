"""The C ABI library: builds, loads, exports what include/mi_inverse.h declares,
and validates arguments before touching a GPU.  CPU only."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from matrixinversion_gb300 import _lib, build

    build.build()
    return _lib.load()


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(mi_\w+)\s*\(", text))
    return syms


def test_exports_every_declared_symbol(lib):
    from matrixinversion_gb300 import build

    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True, check=True)
    exported = set(re.findall(r" T (mi_\w+)", out.stdout))
    declared = declared_symbols()
    assert declared, "no declarations found"
    assert declared <= exported, declared - exported
    for s in declared:
        assert hasattr(lib, s)


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "mi_inverse.h"\nint main(void){return mi_abi_version()==MI_ABI_VERSION?0:1;}\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-c",
                    str(src), "-o", str(tmp_path / "t.o")], check=True)


def test_query_and_errors_without_gpu(lib):
    from matrixinversion_gb300 import _lib

    assert lib.mi_abi_version() == 1
    lanes, mpw, smem, tpb = (ctypes.c_int() for _ in range(4))
    # n <= 15: one thread per matrix, staged through shared memory except at
    # n = 2, where each thread moves its matrix with 16-byte copies; larger n:
    # lane groups
    for n, want, staged in ((1, 1, True), (2, 1, False), (4, 1, True), (5, 1, True), (8, 1, True), (12, 1, True),
                            (15, 1, True), (16, 8, True), (17, 16, True), (32, 16, True)):
        assert lib.mi_query_config(n, ctypes.byref(lanes), ctypes.byref(mpw), ctypes.byref(smem),
                                   ctypes.byref(tpb)) == 0
        assert lanes.value == want and mpw.value == 32 // want and (smem.value > 0) == staged, n
    assert lib.mi_query_config(0, None, None, None, None) == _lib.MI_ERR_INVALID_VALUE
    assert lib.mi_query_config(33, None, None, None, None) == _lib.MI_ERR_INVALID_VALUE
    # argument checks return before any CUDA call
    inv = lib.mi_inverse_f32
    assert inv(None, None, None, 0, 8, 1, None) == _lib.MI_OK               # empty batch
    assert inv(None, None, None, 5, 8, 1, None) == _lib.MI_ERR_NULL_POINTER
    assert inv(None, None, None, 5, 0, 1, None) == _lib.MI_ERR_INVALID_VALUE
    assert inv(None, None, None, 5, 33, 1, None) == _lib.MI_ERR_INVALID_VALUE
    assert inv(None, None, None, -1, 8, 1, None) == _lib.MI_ERR_INVALID_VALUE
    assert inv(None, None, None, 5, 8, 7, None) == _lib.MI_ERR_INVALID_VALUE
    assert inv(ctypes.c_void_p(0x1002), None, None, 5, 8, 1, None) == _lib.MI_ERR_MISALIGNED
    assert lib.mi_inverse_cfg_f32(None, None, None, 5, 8, 1, -32, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert b"invalid" in lib.mi_error_string(_lib.MI_ERR_INVALID_VALUE)


def test_python_surface_rejects_host_tensors():
    import torch

    import matrixinversion_gb300 as mi

    with pytest.raises(TypeError):
        mi.batched_inverse(torch.zeros(2, 4, 4), True)        # no host implementation
    assert mi.pivot_mode(True) == 1 and mi.pivot_mode(False) == 0
    assert mi.pivot_mode("partial") == 3 and mi.pivot_mode("reference_serial") == 2
    with pytest.raises(ValueError):
        mi.pivot_mode("lapack")
