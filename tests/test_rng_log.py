"""dmd_log (csrc/dmd_rng.h), the logarithm every ghost draw goes through
(the exponential inter-ghost time and the Marsaglia polar velocities of
code/main.F90:408-419,997-1121), against the logarithm in extended
precision over 1.02e7 inputs of the ghost-draw range (0, 1): uniform 53-bit
draws, a log-uniform spread down to 2^-53, and the 1e5 doubles on each side
of 1.  Bound: 2.5 ulp of the double result (measured: 2.0).  The GPU's
dmd_log must give the host's bits."""
import ctypes as C

import numpy as np
import pytest

ULP_BOUND = 2.5


def _inputs():
    rng = np.random.default_rng(1)
    n = 10_000_000
    return np.concatenate([rng.integers(1, 2**53, n, dtype=np.int64).astype(np.float64) * 2.0**-53,
                           2.0 ** rng.uniform(-53, 0, n // 10),
                           1.0 - np.arange(1, 100001) * 2.0**-53, 1.0 + np.arange(1, 100001) * 2.0**-52])


def _host_log(x):
    from oracle.oracle import lib
    L = lib()
    L.ora_log_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    y = np.empty_like(x)
    L.ora_log_many(x.ctypes.data, y.ctypes.data, len(x))
    return y


def test_dmd_log_error_bound(built):
    if np.finfo(np.longdouble).nmant < 60:
        pytest.skip("needs an extended-precision long double for the reference logarithm")
    x = _inputs()
    y = _host_log(x)
    ref = np.log(x.astype(np.longdouble))
    ulp = np.spacing(np.abs(ref.astype(np.float64))).astype(np.longdouble)
    err = np.abs((y.astype(np.longdouble) - ref) / ulp)
    assert float(err.max()) <= ULP_BOUND, (float(err.max()), x[np.argmax(err)])
    assert np.all(y[x < 1.0] < 0.0) and np.all(y[x > 1.0] > 0.0)


@pytest.mark.gpu
def test_dmd_log_device_equals_host(built):
    from test_known_answers import _harness
    x = _inputs()
    L = _harness()
    L.ka_log_many.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong]
    y = np.empty_like(x)
    assert L.ka_log_many(x.ctypes.data, y.ctypes.data, len(x)) == 0
    assert np.array_equal(y, _host_log(x))
