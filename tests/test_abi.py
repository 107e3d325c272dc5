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


C_CALLER = r"""
#include <stdio.h>
#include "mi_inverse.h"

int main(void) {
    int form, lanes, mpw, tpb;
    if (mi_abi_version() != MI_ABI_VERSION) return 2;
    if (mi_query_launch(32, MI_PIVOT_PARTIAL, 1000000, 0, &form, &lanes, &mpw, &tpb) != MI_OK) return 3;
    printf("%d %d %d %d\n", form, lanes, mpw, tpb);
    /* argument errors come back as status codes, before any CUDA call */
    if (mi_inverse_f32(NULL, NULL, NULL, 4, 8, MI_PIVOT_REFERENCE, NULL) != MI_ERR_NULL_POINTER) return 4;
    if (mi_inverse_f32(NULL, NULL, NULL, 4, 33, MI_PIVOT_REFERENCE, NULL) != MI_ERR_INVALID_VALUE) return 5;
    printf("%s\n", mi_error_string(MI_ERR_NULL_POINTER));
    return 0;
}
"""


def test_c_caller_links_and_runs_without_gpu(lib, tmp_path):
    """A plain C program includes the header, links libmi_inverse and runs the
    calls that need no device."""
    from matrixinversion_gb300 import build

    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), "-L", build.LIBDIR, "-lmi_inverse", "-Wl,-rpath," + build.LIBDIR], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, (out.returncode, out.stderr)
    first, second = out.stdout.splitlines()[:2]
    assert first == "3 16 2 128"            # whole rows per lane, 16 lanes, 2 matrices per warp, 4 warps
    assert "null" in second


def test_query_and_errors_without_gpu(lib):
    from matrixinversion_gb300 import _lib

    assert lib.mi_abi_version() == 2
    lanes, mpw, smem, tpb = (ctypes.c_int() for _ in range(4))
    # n <= 15: one thread per matrix, staged through shared memory except at
    # n = 2, where each thread moves its matrix with 16-byte copies; larger n:
    # lane groups
    for n, want, staged in ((1, 1, True), (2, 1, False), (4, 1, True), (5, 1, True), (8, 1, True), (12, 1, True),
                            (15, 1, True), (16, 8, True), (17, 16, True), (32, 8, True)):
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


def test_query_launch_reports_the_form_each_call_runs(lib):
    """mi_query_launch follows the contiguous launch's choice of kernel form."""
    import matrixinversion_gb300 as mi
    from matrixinversion_gb300 import _lib

    def q(n, pivot, batch, tpb=0):
        r = mi.query_launch(n, pivot, batch, tpb)
        return r["form"], r["lanes_per_matrix"], r["matrices_per_warp"], r["threads_per_block"], r["knob"]

    # n <= 8: one thread per matrix at any batch, 4 warps per block
    for pivot in ("none", "reference", "reference_serial", "partial"):
        assert q(8, pivot, 10) == ("thread", 1, 32, 128, False)
        assert q(1, pivot, 10**6, 256) == ("thread", 1, 32, 128, False)
    # n = 9..15: one thread per matrix on large batches (2 warps per block up
    # to n = 13, 1 above), lane groups below the measured crossover
    assert q(12, "reference", 10**6) == ("thread", 1, 32, 64, False)
    assert q(15, "none", 12288) == ("thread", 1, 32, 32, False)
    assert q(12, "reference", 12287, 64) == ("lanes", 8, 4, 64, True)
    assert q(12, "partial", 4096) == ("thread", 1, 32, 64, False)
    assert q(12, "partial", 4095, 32) == ("lanes", 16, 2, 32, True)
    # the knob as mi_inverse_cfg_f32 resolves it: 0 = installed entry,
    # rounded up to a warp multiple, capped at 256
    assert q(20, "reference", 1000, 65)[3] == 96
    assert q(20, "reference", 1000, 300)[3] == 256
    assert q(20, "reference", 1000, 0)[3] == lib_tuned(lib, 20, 1)
    # partial pivoting: whole rows per lane at n = 16..32, eight lanes per
    # matrix (four matrices per warp) at n = 17..24, sixteen elsewhere
    for n in (16, 25, 28, 29, 30, 31, 32):
        assert q(n, "partial", 10**6, 64) == ("rows", 16, 2, 128, False), n
    for n in (17, 18, 20, 21, 24):
        assert q(n, "partial", 10**6, 64) == ("rows", 8, 4, 128, False), n
    # n = 32 without partial pivoting: eight lanes per matrix, four matrices per warp
    assert q(32, "reference", 10**6, 128) == ("lanes", 8, 4, 128, True)
    assert q(32, "none", 10, 512) == ("lanes", 8, 4, 256, True)
    # argument errors
    for bad in ((0, 1, 10, 0), (33, 1, 10, 0), (8, 4, 10, 0), (8, -1, 10, 0), (8, 1, -1, 0), (8, 1, 10, -32)):
        assert lib.mi_query_launch(*bad, None, None, None, None) == _lib.MI_ERR_INVALID_VALUE, bad


def lib_tuned(lib, n, pivot):
    v = ctypes.c_int()
    assert lib.mi_get_launch_config(n, pivot, ctypes.byref(v)) == 0
    return v.value


def test_noalloc_and_descriptor_argument_checks_without_gpu(lib):
    """The descriptor entry points validate their arguments before any CUDA call."""
    from matrixinversion_gb300 import _lib

    d = lib.mi_inverse_descr_f32
    big = 1 << 30
    assert d(None, 0, None, None, None, None, None, 0, 0, 0, None, 0, None) == _lib.MI_OK
    assert d(None, 0, None, None, None, None, None, -1, 0, 0, None, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert d(None, -1, None, None, None, None, None, 4, 0, 0, None, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert d(None, big, None, None, None, None, None, 4, 0, 0, None, 0, None) == _lib.MI_ERR_NULL_POINTER
    p = ctypes.c_void_p(0x100000)
    assert d(ctypes.c_void_p(0x100002), big, p, p, p, None, None, 4, 0, 0, p, 1 << 20, None) == _lib.MI_ERR_MISALIGNED
    assert d(p, big, p, p, p, None, None, 4, 0, 0, ctypes.c_void_p(0x100010), 1 << 20, None) == _lib.MI_ERR_MISALIGNED
    need = lib.mi_descr_workspace_bytes(4)
    assert d(p, big, p, p, p, None, None, 4, 0, 0, p, need - 1, None) == _lib.MI_ERR_INVALID_VALUE
    for count in (0, 1, 1000, 262144):
        assert lib.mi_descr_workspace_bytes(count) == (4096 + 4 * count + 255) // 256 * 256
    # the descriptor form: 0 (default) one launch per bucket, c > 0 the
    # single persistent launch with chunks of about c floats
    saved = lib.mi_get_descr_chunk()
    assert saved == 0
    assert lib.mi_set_descr_chunk(-1) == _lib.MI_ERR_INVALID_VALUE and lib.mi_get_descr_chunk() == saved
    assert lib.mi_set_descr_chunk(16384) == _lib.MI_OK and lib.mi_get_descr_chunk() == 16384
    assert lib.mi_set_descr_chunk(saved) == _lib.MI_OK and lib.mi_get_descr_chunk() == saved
    na = lib.mi_inverse_descr_noalloc_f32
    assert na(None, 0, None, None, None, None, None, 0, 0, 0, None) == _lib.MI_OK
    assert na(None, 0, None, None, None, None, None, -5, 0, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert na(p, -1, p, p, p, None, None, 4, 0, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert na(p, big, p, p, p, None, None, _lib.MI_NOALLOC_MAX_COUNT + 1, 0, 0, None) == _lib.MI_ERR_SCRATCH_LIMIT
    # refinement entry points
    assert lib.mi_newton_schulz_f32(None, None, 4, 16, 1, None) == _lib.MI_ERR_INVALID_VALUE
    assert lib.mi_newton_schulz_f32(None, None, 4, 32, 5, None) == _lib.MI_ERR_INVALID_VALUE
    assert lib.mi_newton_schulz_f32(None, None, 0, 32, 1, None) == _lib.MI_OK
    assert lib.mi_newton_schulz_f32(None, None, 4, 32, 1, None) == _lib.MI_ERR_NULL_POINTER
    assert lib.mi_newton_schulz_f32(ctypes.c_void_p(0x100004), p, 4, 32, 1, None) == _lib.MI_ERR_MISALIGNED
    for f in (lib.mi_refine_fp64_f32, lib.mi_refine_df_f32):
        assert f(None, None, None, 4, 4, 33, None) == _lib.MI_ERR_INVALID_VALUE
        assert f(None, None, None, 0, 4, 32, None) == _lib.MI_OK
        assert f(None, None, None, 4, 4, 32, None) == _lib.MI_ERR_NULL_POINTER
    assert lib.mi_refine_df_next_f32(p, p, p, 4, 4, 32, -1.0, p, None) == _lib.MI_ERR_INVALID_VALUE
    f = lib.mi_refine_tc_f32
    assert f(None, None, None, 4, 4, 16, None) == _lib.MI_ERR_INVALID_VALUE          # n = 32 only
    assert f(None, None, None, 0, 4, 32, None) == _lib.MI_OK
    assert f(None, None, None, 4, 4, 32, None) == _lib.MI_ERR_NULL_POINTER
    assert f(ctypes.c_void_p(0x100004), p, p, 4, 4, 32, None) == _lib.MI_ERR_MISALIGNED
    assert lib.mi_refine_tc_next_f32(p, p, p, 4, 4, 32, -1.0, p, None) == _lib.MI_ERR_INVALID_VALUE
    g = lib.mi_refine_tc_flagged_f32
    assert g(p, p, 4, 31, 8.0, 3e-7, p, None) == _lib.MI_ERR_INVALID_VALUE
    assert g(p, p, 4, 32, float("nan"), 3e-7, p, None) == _lib.MI_ERR_INVALID_VALUE
    assert g(p, p, 4, 32, 8.0, -1.0, p, None) == _lib.MI_ERR_INVALID_VALUE
    assert g(None, None, 0, 32, 8.0, 3e-7, None, None) == _lib.MI_OK
    assert g(None, p, 4, 32, 8.0, 3e-7, p, None) == _lib.MI_ERR_NULL_POINTER
    assert g(p, ctypes.c_void_p(0x100008), 4, 32, 8.0, 3e-7, p, None) == _lib.MI_ERR_MISALIGNED
    assert lib.mi_flag_condition_f32(None, None, 4, 0, 8.0, None, None) == _lib.MI_ERR_INVALID_VALUE
    assert lib.mi_flag_condition_f32(None, None, 4, 32, 8.0, None, None) == _lib.MI_ERR_NULL_POINTER


def test_device_error_query_reports_cuda_failure_without_gpu(lib):
    """mi_device_error reads every module's error word through CUDA; with no
    device the first read fails and the call says so (status, message)."""
    import torch

    from matrixinversion_gb300 import _lib

    if torch.cuda.is_available():
        pytest.skip("checks the path without a device")
    v = ctypes.c_int(-7)
    assert lib.mi_device_error(ctypes.byref(v), 1) == _lib.MI_ERR_CUDA
    assert v.value == -7                                   # untouched on failure
    assert b"device error word" in lib.mi_last_cuda_error()


def test_persistent_walk_units_are_relocatable():
    """The single persistent descriptor launch calls walks defined in other
    units: every unit that defines or calls them must be compiled as
    relocatable device code and device-linked, or the library link fails."""
    import glob
    import os

    from matrixinversion_gb300 import build as B

    units = {os.path.basename(p) for p in glob.glob(os.path.join(B.CSRC, "*.cu"))}
    callers = {u for u in units if "MI_PWALK_" in open(os.path.join(B.CSRC, u)).read()}
    assert callers == {"mi_descr_persist.cu", "mi_pwalk_none.cu", "mi_pwalk_reference.cu",
                       "mi_pwalk_reference_serial.cu", "mi_pwalk_partial.cu"}
    assert B.RDC_UNITS == callers
