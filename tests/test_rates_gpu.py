"""The library's rate probes (roofline denominators and the INT8 question):
each returns 0 and positive, plausible rates on the GPU."""
import ctypes as C

import pytest


@pytest.mark.gpu
def test_fp64_rates(gpu_lib):
    from qrdm_gb300 import lib

    out = (C.c_double * 3)()
    assert lib().qrdm_fp64_rates(out, 3) == 0
    fma, dmma884, dmma16816 = out
    # GB300 measured about 1.26 (FMA) and 1.1 (DMMA) TFLOP/s
    assert 0.2 < fma < 100.0 and 0.05 < dmma884 < 100.0 and 0.05 < dmma16816 < 100.0, list(out)


@pytest.mark.gpu
def test_legacy_mma_rates(gpu_lib):
    from qrdm_gb300 import lib

    out = (C.c_double * 2)()
    assert lib().qrdm_legacy_mma_rates(out, 2) == 0
    int8_tops, fp16_tflops = out
    # GB300 measured about 150 TOP/s (INT8) and 600 TFLOP/s (FP16)
    assert 5.0 < int8_tops < 20000.0 and 20.0 < fp16_tflops < 20000.0, list(out)
    assert lib().qrdm_legacy_mma_rates(None, 2) == -1
