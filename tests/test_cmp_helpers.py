"""The integer-pipe compares, selections and sign flips the kernels use in
place of FP64 compares (landslidehysea_gb300/csrc/lsh_fpmath.h,
lsh_scheme.cuh, lsh_passes.cuh) give exactly what the floating-point
expressions give, for every pair of a set of special values: signed zeros,
subnormals, the scheme's thresholds and their neighbours, huge values,
infinities (and NaN where a form keeps NaN semantics).  Host build here,
device build on the GPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from adj_cases import native_lib

HERE = os.path.dirname(os.path.abspath(__file__))


def special_values():
    eps = float(np.finfo(np.float32).eps)
    base = [0.0, 5e-324, 2.2250738585072009e-308, 2.2250738585072014e-308, 1e-300, 2.0 ** -1000, 2.0 ** -54,
            1e-17, 1e-10, 1e-5, eps, 0.5, 0.9999999999999999, 1.0, 1.0000000000000002, 2.0, 3.0, 745.5, 746.0,
            746.5, 1e300, 1.7976931348623157e308, np.inf, 0.136]
    vals = []
    with np.errstate(over="ignore"):
        for b in base:
            vals += [b, np.nextafter(b, np.inf), np.nextafter(b, -np.inf)]
    rng = np.random.default_rng(11)
    vals += list(np.exp(rng.uniform(np.log(1e-320), np.log(1e300), 60)))
    vals += list(rng.standard_normal(20))
    vals = np.array(vals, dtype=np.float64)
    vals = np.concatenate([vals, -vals, [np.nan, -np.nan]])
    return np.ascontiguousarray(np.unique(vals.view(np.uint64)).view(np.float64))


def test_integer_pipe_helpers_equal_the_float_compares_on_the_host():
    v = special_values()
    lib = native_lib("cmp_check")
    assert np.signbit(v[v == 0]).any() and (~np.signbit(v[v == 0])).any()  # both zeros present
    assert np.isnan(v).sum() == 2
    assert lib.cmpc_check(v.ctypes.data, v.size) == 0


@pytest.mark.gpu
def test_integer_pipe_helpers_equal_the_float_compares_on_the_device(gpu_lib, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path / "cmp_check_gpu.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-shared",
                    "-Xcompiler", "-fPIC", os.path.join(HERE, "native", "cmp_check_gpu.cu"), "-o", out], check=True)
    lib = ctypes.CDLL(out)
    lib.cmpc_check_gpu.restype = ctypes.c_int
    lib.cmpc_check_gpu.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    v = special_values()
    per = np.zeros(v.size, dtype=np.int64)
    assert lib.cmpc_check_gpu(v.ctypes.data, v.size, per.ctypes.data) == 0
    bad = {f"{x!r} ({np.float64(x).view(np.uint64):#018x})": int(c) for x, c in zip(v, per) if c}
    assert not bad, bad
