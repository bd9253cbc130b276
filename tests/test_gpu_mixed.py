"""Mixed-precision plan (FP64 sparse grid + FP32 dense bulk) against the FP64 oracle.

Bar (the benchmark spec): |dlnL| <= 1e-2 against the FP64 oracle; the gradient is the
exact gradient of the interpolated model, checked against the oracle's
forward-mode duals to 1e-3 of the gradient norm and against central finite
differences of the mixed lnL itself.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, make_dataset, perturbed, random_prior_theta  # noqa: E402
from tests.test_gpu_plan import DUR, DT, FMAX, FMIN, cuda_detectors, lisa, tianqin  # noqa: E402


@pytest.fixture(scope="module")
def dataset(oracle):
    tc = DUR - 20000.0
    th0 = config0_theta(tc)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle), tianqin(oracle)], th0)
    return g, dets, th0


def engines(g, dets, **kw):
    from pespace_gb300.inference import WhittleLikelihood

    return (WhittleLikelihood(cuda_detectors(g, dets), precision="mixed", reference_frequency=1e-4, **kw),
            WhittleLikelihood(cuda_detectors(g, dets), precision="fp64", reference_frequency=1e-4, **kw))


def test_mixed_lnl_injection_perturbed(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    rng = np.random.default_rng(11)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(15)])
    mixed, fp64 = engines(g, dets[:1], max_batch=16)
    got = mixed.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4).lnl(thetas)
    err = np.abs(got - want)
    assert np.all(mixed.last_status.cpu().numpy() == 0)
    assert err.max() <= 1e-2, err
    # deterministic forward
    assert np.array_equal(got, mixed.log_likelihood_batch(thetas).cpu().numpy())


def test_mixed_prior_batch_cutoff_network(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    rng = np.random.default_rng(2026)
    thetas = random_prior_theta(rng, 48, th0[10])
    mixed, _ = engines(g, dets, max_batch=64, cut_factor=1.2)
    got = mixed.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(thetas, nthreads=8)
    err = np.abs(got - want)
    assert np.median(err) <= 1e-2, np.sort(err)[-5:]
    # loud templates (|lnL - lnL_noise| large) are bounded relatively
    assert np.all(err <= 1e-2 + 1e-7 * np.abs(want)), np.sort(err)[-5:]


def test_mixed_gradient(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    rng = np.random.default_rng(5)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    mixed, _ = engines(g, dets[:1], max_batch=8)
    lnl, grad = mixed.log_likelihood_and_grad(thetas)
    lnl_only = mixed.log_likelihood_batch(thetas)
    assert torch.equal(lnl, lnl_only)
    w_lnl, w_grad = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4).lnl(
        thetas, grad=True, nthreads=8)
    gg = grad.cpu().numpy()
    norm = np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(gg - w_grad) / norm) < 1e-3, (gg, w_grad)
