"""FP32 precision form against the FP64 plain form from the same seed (GPU).

Targets: relative energy drift of the FP32 form within 1e-4 of the FP64 form's,
charge-conservation residual of the FP32 Esirkepov step <= 1e-6 (normalised by
max|rho|/dt, and by max|drho/dt|, the charge the step moves), RMS momentum error
after 10 steps at FP32 rounding level.
"""
import pytest

import pica_gb300 as pg
from pica_gb300 import validate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [pg.SHAPE_TSC, pg.SHAPE_CIC])
def test_fp32_form_errors_against_fp64_form(shape):
    r = validate.compare_forms(n=(16, 16, 16), ppc=32, steps=200, every=10, rms_steps=10, shape=shape)
    assert r["energy_drift_diff_max"] < 1e-4, r
    assert r["charge_residual"] <= 1e-6, r
    assert r["charge_residual_vs_drho"] <= 1e-6, r
    assert r["rms_momentum_error"] is not None and r["rms_momentum_error"] < 1e-5, r
