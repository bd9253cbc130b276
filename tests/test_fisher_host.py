"""Fisher matrix: the oracle's definition checked against the Hessian, and the
host utilities (sampling from N(0, F^-1), angle wrapping) of fisher.py."""

import numpy as np

from tests.helpers import config0_theta, make_dataset
from tests.test_gpu_plan import lisa

DUR = 2.0 ** 16


def test_oracle_fisher_is_minus_hessian_for_noiseless_data(oracle):
    """fisher.py's note: with data equal to the model, F = -Hessian(lnL) at the
    fiducial point (Hessian by central differences of the oracle's exact gradient)."""
    th0 = config0_theta(DUR - 2000.0)
    g, dets = make_dataset(oracle, DUR, 8.0, 1e-4, 0.03, [lisa(oracle)], th0, seed=1)
    _, o, gen, d, p = dets[0]
    h = oracle.Plan(g, [(o, gen, d, p)], 1e-4).model_tdi(0, th0)
    plan = oracle.Plan(g, [(o, gen, h, p)], 1e-4)
    F = plan.fisher(th0[None])[0]
    assert np.array_equal(F, F.T)
    H = np.zeros((11, 11))
    for k in range(11):
        e = 1e-6 if k in (0, 4) else 1e-6 * max(abs(th0[k]), 1.0)
        tp, tm = th0.copy(), th0.copy()
        tp[k] += e
        tm[k] -= e
        H[:, k] = (plan.lnl(tp[None], grad=True)[1][0] - plan.lnl(tm[None], grad=True)[1][0]) / (2 * e)
    s = np.sqrt(np.diag(F))
    assert np.max(np.abs((F + H) / np.outer(s, s))) < 1e-4
    assert np.all(np.linalg.eigvalsh(F / np.outer(s, s)) > 0)


def test_sample_from_fisher_covariance():
    from pespace_gb300.inference import sample_from_fisher

    rng = np.random.default_rng(3)
    A = rng.normal(size=(5, 5))
    F = A @ A.T + 5 * np.eye(5)
    F = F * np.outer([1e6, 1.0, 1e-3, 10.0, 1e4], [1e6, 1.0, 1e-3, 10.0, 1e4])  # mixed units
    x = sample_from_fisher(F, 200000, rkey_seed=7)
    C = np.linalg.inv(F)
    s = np.sqrt(np.diag(C))
    assert np.max(np.abs((np.cov(x.T) - C) / np.outer(s, s))) < 0.02
    assert np.array_equal(x[:10], sample_from_fisher(F, 10, rkey_seed=7)[:10])


def test_wrap_angle_params():
    from pespace_gb300.inference import wrap_angle_params

    s = {"ecliptic_longitude": np.array([-0.5, 7.0]), "ecliptic_latitude": np.array([1.7, -2.0]),
         "inclination": np.array([-0.3, 3.5]), "polarization": np.array([4.0, -1.0]),
         "reference_phase": np.array([6.5, -0.1]), "chirp_mass": np.array([1.0, 2.0])}
    w = wrap_angle_params(s)
    assert np.all((w["ecliptic_longitude"] >= 0) & (w["ecliptic_longitude"] < 2 * np.pi))
    assert np.all(np.abs(w["ecliptic_latitude"]) <= np.pi / 2)
    assert np.allclose(w["ecliptic_latitude"], [np.pi - 1.7, -np.pi + 2.0])
    assert np.allclose(w["inclination"], [0.3, 2 * np.pi - 3.5])
    assert np.all((w["polarization"] >= 0) & (w["polarization"] < np.pi))
    assert w["chirp_mass"] is s["chirp_mass"]
    assert np.array_equal(s["ecliptic_longitude"], [-0.5, 7.0])  # input untouched


def test_fiducial_parameter_forms():
    """Arrays, lists and tensors (any device) give the same (B, 11) rows."""
    import torch

    from pespace_gb300.inference.fisher import _as_theta

    row = np.linspace(0.1, 1.1, 11)
    for x in (row, list(row), torch.as_tensor(row)):
        th, single = _as_theta(x)
        assert single and th.shape == (1, 11) and th.dtype == torch.float64
        assert np.array_equal(th[0].numpy(), row)
    th, single = _as_theta(torch.as_tensor(np.stack([row, 2 * row])))
    assert not single and th.shape == (2, 11)
