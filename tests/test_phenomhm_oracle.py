"""IMRPhenomHM restatement of the oracle (London et al. 2018): parity against
reference code is unpinned (the reference's waveforms come from the absent
tiwave/ripple packages), so these are the model's own identities.

* the (2,2) mode is IMRPhenomD's, bit for bit;
* t_lm(f) = dPsi_lm/df / (2 pi) (central differences);
* Psi_lm and A_lm are C1 across the frequency-map corners;
* below the inspiral corners, Psi_lm(f) = (m/2) Psi_22(2f/m) + k pi/2 and
  A_lm(f) = beta_lm A_22(2f/m), beta_lm tending to the leading-order
  post-Newtonian mode ratio as v -> 0;
* each mode's ringdown sits at its own Kerr frequency;
* the spin-weighted spherical harmonics are normalised.
"""

import math

import numpy as np
import pytest

from tests.helpers import config0_theta, random_prior_theta

MODES = ((2, 2), (2, 1), (3, 3), (3, 2), (4, 4), (4, 3))


def _msec(th):
    eta = th[1] / (1 + th[1]) ** 2
    return math.exp(th[0]) * eta ** -0.6 * 4.925490947641266978197229498498379006e-6


def thetas():
    rng = np.random.default_rng(8)
    return [config0_theta(4e6)] + list(random_prior_theta(rng, 5, 4e6))


@pytest.mark.parametrize("k", range(6))
def test_22_is_phenomd_and_time_identity(oracle, k):
    for th in thetas():
        ms = _msec(th)
        f = np.geomspace(2e-4, 0.3, 3001) / ms  # Mf from 2e-4 to 0.3
        hp, hc, tf, A, P, info = oracle.phenomhm(th, f, 1e-4)
        if k == 0:
            hpd, hcd, tfd, _, Ad, Pd = oracle.phenomd(th, f, 1e-4, amp_psi=True)
            np.testing.assert_array_equal(A[0], Ad)
            np.testing.assert_array_equal(P[0], Pd)
            np.testing.assert_array_equal(tf[0], tfd)
            np.testing.assert_allclose(hp[0], hpd, rtol=0, atol=1e-15 * np.abs(hpd).max())
            np.testing.assert_allclose(hc[0], hcd, rtol=0, atol=1e-15 * np.abs(hcd).max())
        # t(f) = dPsi/df / 2pi by central differences, away from the map corners
        live = A[k] > 0
        fl = f[live][5:-5:7]
        h = 1e-6 * fl
        _, _, tfl, _, _, _ = oracle.phenomhm(th, fl, 1e-4)
        _, _, _, _, Pp, _ = oracle.phenomhm(th, fl + h, 1e-4)
        _, _, _, _, Pm, _ = oracle.phenomhm(th, fl - h, 1e-4)
        corners = np.array([info[k, 2], info[k, 3]]) / ms
        far = np.min(np.abs(fl[:, None] - corners[None, :]), axis=1) > 10 * h
        fd = (Pp[k] - Pm[k]) / (2 * h) / (2 * math.pi)
        scale = np.abs(tfl[k][far]) + ms
        assert np.max(np.abs(fd[far] - tfl[k][far]) / scale) < 1e-5


@pytest.mark.parametrize("k", range(1, 6))
def test_continuity_at_corners(oracle, k):
    for th in thetas():
        ms = _msec(th)
        _, _, _, _, _, info = oracle.phenomhm(th, np.array([1e-3]), 1e-4)
        # the amplitude-map inspiral corner and the phase-map ringdown corner
        for corner, what in ((info[k, 2], "amp"), (info[k, 3], "phase")):
            fc = corner / ms
            eps = 1e-9 * fc
            f = np.array([fc - eps, fc + eps, fc - 2e-4 * fc, fc + 2e-4 * fc])
            _, _, tf, A, P, _ = oracle.phenomhm(th, f, 1e-4)
            if A[k, 0] == 0:
                continue  # above the cut
            assert abs(A[k, 1] - A[k, 0]) <= 1e-6 * A[k, 0], (what, A[k])
            assert abs(P[k, 1] - P[k, 0]) <= 1e-6 * (1 + abs(P[k, 0])), (what, P[k])
            # C1 phase: t(f) continuous
            assert abs(tf[k, 1] - tf[k, 0]) <= 1e-5 * (abs(tf[k, 0]) + ms), (what, tf[k])
            if what == "amp":  # the amplitude is C1 across its map's corners
                e = 1e-6 * fc
                fa = np.array([fc - 3 * e, fc - e, fc + e, fc + 3 * e])
                _, _, _, Aa, _, _ = oracle.phenomhm(th, fa, 1e-4)
                left, right = (Aa[k, 1] - Aa[k, 0]) / (2 * e), (Aa[k, 3] - Aa[k, 2]) / (2 * e)
                assert abs(right - left) <= 1e-3 * abs(left), (left, right)


@pytest.mark.parametrize("k", range(1, 6))
def test_inspiral_scaling_and_pn_ratio(oracle, k):
    l, m = MODES[k]
    th = config0_theta(4e6).copy()
    th[2], th[3] = 0.0, 0.0  # non-spinning: the spin term of (2,1) is off
    ms = _msec(th)
    q = th[1]
    eta, dlt = q / (1 + q) ** 2, (q - 1) / (q + 1)
    Mf = np.geomspace(1e-5, 3e-3, 50)
    f = Mf / ms
    _, _, _, A, P, info = oracle.phenomhm(th, f, 1e-4)
    assert np.all(Mf < info[k, 2])
    _, _, _, A22, P22, _ = oracle.phenomhm(th, 2 * f / m, 1e-4)
    kq = {(2, 1): 1, (3, 3): 3, (3, 2): 0, (4, 4): 2, (4, 3): 3}[(l, m)]
    np.testing.assert_allclose(P[k], 0.5 * m * P22[0] + kq * math.pi / 2, rtol=1e-12, atol=1e-9)
    beta = A[k] / A22[0]
    v = (2 * math.pi * Mf / m) ** (1 / 3)
    lead = {(2, 1): dlt * v / 3, (3, 3): 0.75 * math.sqrt(15 / 14) * dlt * v,
            (3, 2): math.sqrt(5 / 7) / 3 * v ** 2 * (1 - 3 * eta), (4, 4): 8 / 9 * math.sqrt(5 / 7) * v ** 2 * (1 - 3 * eta),
            (4, 3): 9 / (4 * math.sqrt(70)) * dlt * v ** 3 * (1 - 2 * eta)}[(l, m)] * math.sqrt(2 / m)
    rel = np.abs(beta / lead - 1)
    assert rel[0] < 5 * v[0] ** 2 and rel[-1] < 0.5  # leading order as v -> 0, corrections O(v^2)


def test_ringdown_frequencies(oracle):
    """Each mode's ringdown sits at its own Kerr frequency: fRD_lm ordered as
    the quasi-normal modes are (l = m modes rising with l, (l, l-1) below
    (l, l)), and the ringdown map's slope Rholm = fRD_22 / fRD_lm."""
    for th in thetas():
        _, _, _, _, _, info = oracle.phenomhm(th, np.array([1e-3]), 1e-4)
        frd = dict(zip(MODES, info[:, 0]))
        assert frd[(2, 1)] < frd[(2, 2)] < frd[(3, 2)] < frd[(3, 3)] and frd[(4, 3)] < frd[(4, 4)]
        assert frd[(3, 3)] < frd[(4, 4)]
        np.testing.assert_allclose(info[:, 1], info[0, 0] / info[:, 0], rtol=1e-14)


def test_spherical_harmonics_and_polarisation_factors(oracle):
    """The s = -2 harmonics (Wigner d^l_{m,2}) are normalised, and the oracle's
    hp = P_lm h_lm, hc = i C_lm h_lm use P, C = [(-1)^l Y_{l,-m} +- Y_lm] / (2 N)."""
    c = np.linspace(-1, 1, 20001)
    for l, m in MODES + ((2, -2), (2, -1), (3, -3), (3, -2), (4, -4), (4, -3)):
        y = np.array([_sylm(l, m, ci) for ci in c])
        norm = 2 * math.pi * np.trapezoid(y ** 2, c)
        assert abs(norm - 1) < 1e-6, (l, m, norm)
    y22 = np.array([_sylm(2, 2, ci) for ci in c[::1000]])
    np.testing.assert_allclose(y22, math.sqrt(5 / (64 * math.pi)) * (1 + c[::1000]) ** 2, rtol=1e-12, atol=1e-15)
    nrm = math.sqrt(5 / (16 * math.pi))
    for ci in (-0.9, -0.3, 0.2, 0.75):
        th = config0_theta(4e6).copy()
        th[5] = ci
        hp, hc, _, A, P, _ = oracle.phenomhm(th, np.array([1e-3]), 1e-4)
        for k, (l, m) in enumerate(MODES):
            h = A[k] * np.exp(-1j * P[k])
            sg = (-1) ** l
            Pf = (sg * _sylm(l, -m, ci) + _sylm(l, m, ci)) / (2 * nrm)
            Cf = (sg * _sylm(l, -m, ci) - _sylm(l, m, ci)) / (2 * nrm)
            np.testing.assert_allclose(hp[k], Pf * h, rtol=1e-12, atol=1e-30)
            np.testing.assert_allclose(hc[k], 1j * Cf * h, rtol=1e-12, atol=1e-30)


def _sylm(l, m, ci):
    ch, sh = math.sqrt(0.5 * (1 + ci)), math.sqrt(max(0.0, 0.5 * (1 - ci)))
    s = 0.0
    fa = math.factorial
    for k in range(0, l + m + 1):
        if l + m - k < 0 or l - 2 - k < 0 or k + 2 - m < 0:
            continue
        s += ((-1) ** k * math.sqrt(fa(l + m) * fa(l - m) * fa(l + 2) * fa(l - 2))
              / (fa(l + m - k) * fa(l - 2 - k) * fa(k) * fa(k + 2 - m)) * ch ** (2 * l + m - 2 * k - 2)
              * sh ** (2 * k + 2 - m))
    return math.sqrt((2 * l + 1) / (4 * math.pi)) * s


def test_polarisation_factors_of_22(oracle):
    th = config0_theta(4e6)
    f = np.array([1e-3, 3e-3])
    hp, hc, _, A, P, _ = oracle.phenomhm(th, f, 1e-4)
    h22 = A[0] * np.exp(-1j * P[0])
    np.testing.assert_allclose(hp[0], 0.5 * (1 + th[5] ** 2) * h22, rtol=1e-13)
    np.testing.assert_allclose(hc[0], -1j * th[5] * h22, rtol=1e-13)
