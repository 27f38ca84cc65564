"""The FP32 Newton iteration of the pressure relaxation (ffv_m5_fp32.cu, relax_face_df) takes
e = (1 + x)^a - 1, a = -1/gamma, from a binomial series in Horner form when |x| <= 1/32, with
the ratios (a - j) / (j + 1), j = 1..6, that ffv_api.cu stores per material.  This restates the
series in FP32 (fused multiply-adds rounded once) and checks it against the exact value for
the stiffened-gas exponents of the configurations, over the whole interval."""
import numpy as np
import pytest


def series_f32(x: np.ndarray, gamma: float) -> np.ndarray:
    f32 = np.float32
    a = -1.0 / gamma
    cb = [f32((a - j) / (j + 1.0)) for j in range(1, 7)]
    x = x.astype(np.float32)

    def fma(p, q, r):  # one rounding, as fmaf
        return (p.astype(np.float64) * q.astype(np.float64) + np.float64(r)).astype(np.float32)

    t = fma(cb[5] * x, np.ones_like(x), 1.0)
    for j in (4, 3, 2, 1, 0):
        t = fma((cb[j] * x).astype(np.float32), t, 1.0)
    ig = f32(1.0 / gamma)
    return ((-ig * x).astype(np.float32) * t).astype(np.float32)


@pytest.mark.parametrize("gamma", [1.0001, 1.4, 3.5, 4.4])
def test_binomial_series_within_two_ulp(gamma):
    x = np.concatenate([np.linspace(-1 / 32, 1 / 32, 100001),
                        np.geomspace(1e-12, 1 / 32, 2000), -np.geomspace(1e-12, 1 / 32, 2000)])
    x = x.astype(np.float32)
    exact = np.expm1(-np.log1p(x.astype(np.float64)) / gamma)
    got = series_f32(x, gamma).astype(np.float64)
    ok = exact != 0.0
    rel = np.abs(got[ok] - exact[ok]) / np.abs(exact[ok])
    assert rel.max() < 2.0 * 2.0 ** -23, rel.max()
