"""Identities and conventions of the reference that its own notebooks check
(orbit_model.ipynb, psd.ipynb, likelihood.ipynb), asserted here on the oracle
and on the host-side noise models (CPU)."""

import numpy as np
import pytest

from oracle import fdpath

YEAR = 365.25 * 86400.0


@pytest.mark.parametrize("kind", ["heliocentric", "geocentric"])
def test_orbit_unit_vectors_match_positions(kind):
    """n1 = (x3 - x2)/L, n2 = (x1 - x3)/L, n3 = (x2 - x1)/L and |n_i| = 1 over a
    year (orbit.py:18-23; the reference's notebook finds 8.8e-15 and 2.0e-13)."""
    fdpath.build()
    if kind == "heliocentric":
        desc = fdpath.heliocentric(2.5e9, 0.3, -np.pi / 9)
    else:
        desc = fdpath.geocentric(np.sqrt(3.0) * 1e8, 0.4, 1.1)
    t = np.random.default_rng(5).uniform(0.0, YEAR, 2000)
    v = fdpath.orbit_vectors(desc, t)
    n, x = v[:, 0:3, :], v[:, 3:6, :]
    L = desc.arm_sec
    want = np.stack([x[:, 2] - x[:, 1], x[:, 0] - x[:, 2], x[:, 1] - x[:, 0]], axis=1) / L
    assert np.max(np.abs(n - want)) < (1e-13 if kind == "heliocentric" else 1e-12)
    assert np.max(np.abs(np.linalg.norm(n, axis=-1) - 1.0)) < 1e-13


@pytest.mark.parametrize("model", ["LISA_SciRDv1", "Taiji_TDC", "Tianqin_GWSpace"])
@pytest.mark.parametrize("generation", ["1.5", "2.0"])
def test_psd_channel_symmetries(model, generation):
    """A and E share one PSD, and so do X, Y and Z (psd.ipynb cell 5)."""
    from pespace_gb300.detector.noise import available_noise_models

    f = np.geomspace(1e-5, 0.5, 4001)
    psd = available_noise_models[model](f, ("A", "E", "T", "X", "Y", "Z"), False, generation)
    assert np.array_equal(psd["A"], psd["E"])
    assert np.array_equal(psd["X"], psd["Y"]) and np.array_equal(psd["X"], psd["Z"])
    assert np.all(psd["A"] > 0) and np.all(psd["T"] >= 0)


@pytest.mark.parametrize("seed", [2026, 7])
def test_noise_only_lnl_normalisation(seed):
    """The reference's noise realisation (tdi.py:896-916) has E|n|^2 = S/(2 df)
    per bin, and its lnL is -2 df sum |d - h|^2 / S (likelihood_ti.py:58-68):
    noise-only data give -1 per bin and channel at h = 0 (each term is an
    exponential variate of mean 1), which the oracle reproduces."""
    fdpath.build()
    g = fdpath.grid(2.0 ** 20, 8.0, 1e-4, 0.03)
    psd = fdpath.psd(g["freqs"], "AET", False, "1.5", **fdpath.PSD_PRESETS["LISA_SciRDv1"])
    n = fdpath.noise_realization(g, psd, "AET", seed)
    d = np.stack([n[c] for c in "AET"])
    S = np.stack([psd[c] for c in "AET"])
    lnl = fdpath.whittle(d, np.zeros_like(d), S, g["df"])
    m = d.size
    assert abs(lnl + m) < 5.0 * np.sqrt(m), (lnl, m)
