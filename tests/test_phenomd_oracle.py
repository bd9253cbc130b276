"""Self-consistency of the IMRPhenomD restatement (no reference pins its values):
region joins are C1-continuous, t(f) = (1/2pi) dPsi/df, t(f_peak) = 0, the
amplitude tends to the leading-order SPA amplitude at low frequency."""

import numpy as np
import pytest

from tests.helpers import config0_theta


@pytest.mark.parametrize("q,c1,c2", [(2.0, 0.5, -0.3), (1.0, 0.0, 0.0), (8.0, 0.9, -0.9), (3.0, -0.95, 0.95)])
def test_phenomd_continuity_and_time(oracle, q, c1, c2):
    th = config0_theta(0.0)
    th[1], th[2], th[3] = q, c1, c2
    _, _, _, info = oracle.phenomd(th, np.array([1e-3]), 1e-4)
    Ms = info["M_sec"]
    for fj in (0.014, 0.018, info["fpeak"], 0.5 * info["fRD"]):
        f = np.array([fj * (1 - 1e-10), fj * (1 + 1e-10)]) / Ms
        hp, hc, tf, _ = oracle.phenomd(th, f, 1e-4)
        assert abs(abs(hp[1]) / abs(hp[0]) - 1) < 1e-7
        assert abs(np.angle(hp[1] / hp[0])) < 1e-6
        assert abs(tf[1] - tf[0]) < 1e-5 * max(1.0, abs(tf[0]))
    # t(f) = dPsi/df / 2pi with h ~ e^{-i Psi}
    f = np.geomspace(2e-4 / Ms, 0.15 / Ms, 60)
    eps = 1e-7
    hp1, _, tf, _ = oracle.phenomd(th, f * (1 - eps), 1e-4)
    hp2, _, _, _ = oracle.phenomd(th, f * (1 + eps), 1e-4)
    _, _, tf0, _ = oracle.phenomd(th, f, 1e-4)
    dpsi = -np.angle(hp2 / hp1) / (2 * eps * f)
    np.testing.assert_allclose(dpsi / (2 * np.pi), tf0, rtol=2e-4, atol=2e-4 * Ms)
    _, _, tpk, _ = oracle.phenomd(th, np.array([info["fpeak"] / Ms]), 1e-4)
    assert abs(tpk[0]) < 1e-9 * Ms


def test_phenomd_low_frequency_limit(oracle):
    th = config0_theta(0.0)
    _, _, _, info = oracle.phenomd(th, np.array([1e-3]), 1e-4)
    Ms = info["M_sec"]
    f = np.array([1e-6 / Ms])
    hp, hc, tf, _ = oracle.phenomd(th, f, 1e-4)
    mc = np.exp(th[0]) * oracle.MTSUN_SI
    dl = np.exp(th[4]) * 1e6 * oracle.PC_SI / oracle.C_SI
    a_lo = np.sqrt(5 / 24) * np.pi ** (-2 / 3) * mc ** (5 / 6) * f ** (-7 / 6) / dl
    h22 = abs(hp[0]) / (0.5 * (1 + th[5] ** 2))
    assert abs(h22 / a_lo[0] - 1) < 2e-3
    # leading-order time to merger
    eta = th[1] / (1 + th[1]) ** 2
    t_lo = -5 / (256 * eta) * Ms * (np.pi * Ms * f[0]) ** (-8 / 3)
    assert abs(tf[0] / t_lo - 1) < 5e-3
