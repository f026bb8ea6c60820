"""The engine's exponential (ldo_math.h) on the host: accuracy and special
values.  tests/test_gpu_scaffold.py checks that the GPU gives the same bits."""
import numpy as np

from oracle_lib import engine_exp


def test_engine_exp_within_one_ulp():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-700, 700, 300000), rng.uniform(-30, 30, 300000), rng.normal(0, 1e-4, 10000)])
    y = engine_exp(x)
    ref = np.exp(x)
    err = np.abs(y - ref) / np.spacing(ref)
    assert err.max() <= 1.5   # numpy's exp is itself within about half a unit


def test_engine_exp_special_values():
    y = engine_exp(np.array([0.0, -0.0, 710.0, -746.0, np.inf, -np.inf, np.nan, 1.0]))
    assert y[0] == 1.0 and y[1] == 1.0
    assert y[2] == np.inf and y[3] == 0.0
    assert y[4] == np.inf and y[5] == 0.0
    assert np.isnan(y[6])
    assert abs(y[7] - np.e) <= np.spacing(np.e)
