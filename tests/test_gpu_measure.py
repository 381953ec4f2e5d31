"""The multiply-rate probe behind the integer-multiply roofline (probe/mulrate.cu, built into its own
librnsckks_probe.so, not the library): five positive rates, none above the four warp instructions an SM can
issue per cycle, the 32-bit IMAD the fastest."""
import ctypes

import pytest


@pytest.mark.gpu
def test_multiply_rates_are_sane(pkg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from rnsckks_gb300._lib import probe_lib
    rates = (ctypes.c_double * 5)()
    assert probe_lib().rc_measure_multiply_rates(rates, None) == 0
    r = list(rates)
    assert all(0 < x <= 4.0 for x in r)
    assert r[1] == max(r)  # 32-bit IMAD
    assert r[4] < r[3] < r[0]  # __umul64hi < 64-bit low product < IMAD.WIDE


def test_probe_is_not_in_the_library(pkg):
    """The library exports product entry points only; the probe lives in its own shared object."""
    pkg.build()
    assert not hasattr(pkg.lib(), "rc_measure_multiply_rates")
    from rnsckks_gb300._lib import probe_lib
    assert hasattr(probe_lib(), "rc_measure_multiply_rates")
