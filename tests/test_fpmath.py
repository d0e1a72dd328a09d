"""The elementary functions shared by the CUDA kernels and the CPU oracle
(landslidehysea_gb300/csrc/lsh_fpmath.h) against the C library's: a few ulp
over their whole input range, and the exact end values."""
import numpy as np
import pytest


def ulp_err(y, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return np.abs(y - ref) / np.spacing(np.abs(ref))


@pytest.fixture(scope="module")
def xs():
    rng = np.random.default_rng(3)
    return rng


def test_exp_neg(oracle, xs):
    x = np.concatenate([np.exp(xs.uniform(np.log(2.0 ** -54), np.log(700.0), 200000)),
                        xs.uniform(0, 40, 100000), [2.0 ** -54, 1e-10, 0.5, 1.0, 50.0, 700.0]])
    y = oracle.fpmath("exp_neg", x)
    assert np.max(ulp_err(y, np.exp(-x))) <= 4
    z = oracle.fpmath("exp_neg", np.array([0.0, 1e-17, 2.0 ** -55, 746.5, 1e300]))
    assert list(z) == [1.0, 1.0, 1.0, 0.0, 0.0]
    sub = np.array([709.0, 720.0, 740.0, 745.0])   # subnormal results
    assert np.max(np.abs(oracle.fpmath("exp_neg", sub) - np.exp(-sub)) / np.exp(-sub)) < 1e-3


def test_cbrt(oracle, xs):
    x = np.concatenate([np.exp(xs.uniform(np.log(1e-300), np.log(1e300), 200000)), xs.uniform(0, 10, 100000),
                        [1.0, 8.0, 27.0, 1e-310, 4.9e-324]])
    y = oracle.fpmath("cbrt", x)
    # FP32 first guess plus two FP64 Newton steps: at most 3 ulp from numpy's cube root
    assert np.max(ulp_err(y[:-2], np.cbrt(x[:-2]))) <= 3
    assert np.allclose(y[-2:], np.cbrt(x[-2:]), rtol=1e-12, atol=0)
    assert oracle.fpmath("cbrt", np.array([0.0]))[0] == 0.0


def test_log_and_pow(oracle, xs):
    x = np.concatenate([np.exp(xs.uniform(np.log(1e-300), np.log(1e300), 200000)), xs.uniform(0.5, 2.0, 100000)])
    y = oracle.fpmath("log", x)
    ref = np.log(x)
    big = np.abs(ref) > 1e-3
    assert np.max(ulp_err(y[big], ref[big])) <= 4
    assert np.max(np.abs(y - ref)) <= 4e-16 * np.max(np.abs(ref))
    a = xs.uniform(1e-6, 1.0, 100000)
    assert np.max(np.abs(oracle.fpmath("pow1e-3", a) - a ** 1e-3)) <= 4e-16
