"""IMRPhenomHM (six modes) through the FP64 plan against the oracle: lnL at the
injection and perturbed points and on prior draws with the cut at 1.2 times
the largest ringdown frequency (|dlnL| <= 1e-6), the dense A/E/T model per bin
(1e-10 of the per-bin response), a two-detector network, and the gradient
against the oracle's forward-mode dual numbers."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, make_dataset, perturbed, random_prior_theta  # noqa: E402
from tests.test_gpu_plan import DUR, DT, FMAX, FMIN, cuda_detectors, lisa, tianqin  # noqa: E402


def hm_dataset(oracle, dets, th0, seed=2026):
    """Noise plus an IMRPhenomHM injection (oracle model)."""
    g, out = make_dataset(oracle, DUR, DT, FMIN, FMAX, dets, th0, seed=seed)
    # replace the PhenomD injection by the HM one: data = noise + h_HM
    plan_d = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in out], 1e-4)
    plan_hm = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in out], 1e-4, approximant="IMRPhenomHM")
    for i in range(len(out)):
        out[i][3] = out[i][3] - plan_d.model_tdi(i, th0) + plan_hm.model_tdi(i, th0)
    return g, out


@pytest.fixture(scope="module")
def dataset(oracle):
    th0 = config0_theta(DUR - 20000.0)
    g, dets = hm_dataset(oracle, [lisa(oracle), tianqin(oracle)], th0)
    return g, dets, th0


def engine(g, dets, **kw):
    from pespace_gb300.inference import WhittleLikelihood

    return WhittleLikelihood(cuda_detectors(g, dets), precision="fp64", reference_frequency=1e-4,
                             approximant="IMRPhenomHM", **kw)


def oracle_plan(oracle, g, dets, **kw):
    return oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, approximant="IMRPhenomHM", **kw)


def test_hm_lnl_injection_perturbed(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    rng = np.random.default_rng(12)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(5)])
    eng = engine(g, dets[:1], max_batch=8)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle_plan(oracle, g, dets[:1]).lnl(thetas)
    assert np.all(eng.last_status.cpu().numpy() == 0)
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-6)


def test_hm_dense_model_parity(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    eng = engine(g, dets, max_batch=2)
    plan = oracle_plan(oracle, g, dets)
    for d in range(2):
        got = eng.model_tdi(th0, det=d).cpu().numpy()
        want = plan.model_tdi(d, th0)
        mag = np.sqrt(np.sum(np.abs(want) ** 2, axis=0))
        live = mag > 0
        assert np.max(np.abs(got - want)[:, live] / mag[live]) < 1e-10


def test_hm_prior_batch_network_cut(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    thetas = random_prior_theta(np.random.default_rng(2026), 12, th0[10])
    eng = engine(g, dets, max_batch=16, cut_factor=1.2)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle_plan(oracle, g, dets, cut_factor=1.2).lnl(thetas, nthreads=8)
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-6)


def test_hm_gradient(cuda_lib, oracle, dataset):
    g, dets, th0 = dataset
    rng = np.random.default_rng(5)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(2)])
    eng = engine(g, dets[:1], max_batch=4)
    lnl, grad = eng.log_likelihood_and_grad(thetas)
    w_lnl, w_grad = oracle_plan(oracle, g, dets[:1]).lnl(thetas, grad=True, nthreads=8)
    np.testing.assert_allclose(lnl.cpu().numpy(), w_lnl, rtol=1e-11, atol=1e-6)
    scale = np.abs(w_grad) + 1e-9 * np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(grad.cpu().numpy() - w_grad) / scale) < 1e-7


def test_hm_container_and_six_mode_response(cuda_lib, oracle):
    """pes_phenomhm against the oracle's container (mode by mode), and the
    six-mode response through pes_response_links against the oracle's mode sum
    (antenna.py:446-458) within 1e-13 of the per-bin link scale."""
    import torch

    from pespace_gb300 import _lib
    from pespace_gb300.detector.orbit import KaplerianHeliocentric
    from pespace_gb300.waveform import IMRPhenomHM

    g = oracle.grid(DUR, DT, FMIN, FMAX)
    freqs = g["freqs"]
    for th in [config0_theta(DUR - 20000.0)] + list(random_prior_theta(np.random.default_rng(4), 3, DUR - 20000.0)):
        wf = IMRPhenomHM(freqs, 1e-4)
        out = wf.from_theta(th)
        hp = torch.stack([out[m]["plus"] for m in wf.modes]).cpu().numpy()
        hc = torch.stack([out[m]["cross"] for m in wf.modes]).cpu().numpy()
        tf = torch.stack([out[m]["tf"] for m in wf.modes]).cpu().numpy()
        th0 = th.copy()
        th0[10] = 0.0
        ohp, ohc, otf, _, _, _ = oracle.phenomhm(th0, freqs, 1e-4)
        for k in range(6):
            scale = np.abs(ohp[k]).max() + np.abs(ohc[k]).max()
            assert np.max(np.abs(hp[k] - ohp[k])) <= 1e-10 * scale, k
            assert np.max(np.abs(hc[k] - ohc[k])) <= 1e-10 * scale, k
            assert np.max(np.abs(tf[k] - otf[k])) <= 1e-10 * (np.abs(otf[k]).max() + 1.0), k
        # the response of the oracle's container: GPU kernel against the oracle's mode sum
        desc = oracle.heliocentric(2.5e9, 0.0, -np.pi / 9)
        orb = KaplerianHeliocentric(2.5e9, 0.0, -np.pi / 9)
        lam, beta, psi, tc = 1.3, -0.4, 0.9, th[10]
        want = oracle.response_links(desc, freqs, ohp, ohc, otf, lam, beta, psi, tc)
        n = freqs.size
        d_f = torch.as_tensor(freqs, device="cuda")
        d_hp = torch.as_tensor(ohp, device="cuda").contiguous()
        d_hc = torch.as_tensor(ohc, device="cuda").contiguous()
        d_tf = torch.as_tensor(otf, device="cuda").contiguous()
        links = torch.empty((6, n), dtype=torch.complex128, device="cuda")
        lib = _lib.load()
        _lib.check(lib.pes_response_links(orb.to_c(), _lib.ptr(d_f), n, 6, _lib.ptr(d_hp), _lib.ptr(d_hc),
                                          _lib.ptr(d_tf), lam, beta, psi, tc, _lib.ptr(links),
                                          _lib.stream_handle()))
        got = links.cpu().numpy()
        scale = np.sum(np.abs(want), axis=0) + 1e-300
        assert np.max(np.abs(got - want) / scale) < 1e-13


def test_hm_mixed_plan(cuda_lib, oracle, dataset):
    """The mixed plan with the six modes as virtual samples (per-mode sparse
    splines, kinks, anchors and midpoint corrections; the modes summed per bin
    before the residual) against the oracle on the two-detector network:
    |dlnL| <= 1e-2 at the injection, at perturbed points and at prior draws
    with the cut at 1.2 times the largest ringdown frequency.  The mixed
    gradient is refused for IMRPhenomHM (the FP64 plan gives it)."""
    from pespace_gb300 import _lib
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    rng = np.random.default_rng(17)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(5)] + list(random_prior_theta(rng, 10, th0[10])))
    mixed = WhittleLikelihood(cuda_detectors(g, dets), precision="mixed", reference_frequency=1e-4,
                              approximant="IMRPhenomHM", max_batch=16, cut_factor=1.2)
    got = mixed.log_likelihood_batch(thetas).cpu().numpy()
    assert np.all(mixed.last_status.cpu().numpy() == 0)
    want = oracle_plan(oracle, g, dets, cut_factor=1.2).lnl(thetas, nthreads=8)
    err = np.abs(got - want)
    assert np.all(err <= 1e-2), (err, want)
    assert np.array_equal(got, mixed.log_likelihood_batch(thetas).cpu().numpy())  # deterministic
    # every sample re-evaluated (six modes: float-float from the splines, or exactly)
    mixed.refine_all = True
    ff = mixed.log_likelihood_batch(thetas).cpu().numpy()
    work = mixed.last_work(len(thetas))
    assert work["refined_ff"] + work["refined_exact"] == len(thetas)
    assert np.all(np.abs(ff - want) <= 1e-2), (np.abs(ff - want), want)
    mixed.refine_all = False
    with pytest.raises(_lib.PesError):
        mixed.log_likelihood_and_grad(thetas[:2])


def test_hm_mixed_model(cuda_lib, oracle, dataset):
    """The mixed plan's dense six-mode model per bin against the oracle's:
    within 3e-5 of the per-bin response scale (six modes, each with its FP32
    phase and transfer rounding, summed in FP32)."""
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision="mixed", reference_frequency=1e-4,
                            approximant="IMRPhenomHM", max_batch=2)
    plan = oracle_plan(oracle, g, dets)
    for d in range(2):
        got = eng.model_tdi(th0, det=d).cpu().numpy()
        want = plan.model_tdi(d, th0)
        mag = np.sqrt(np.sum(np.abs(want) ** 2, axis=0))
        live = mag > 1e-6 * mag.max()
        assert np.max(np.abs(got - want)[:, live] / mag[live]) < 3e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hm_fisher(cuda_lib, oracle, dataset, precision):
    """IMRPhenomHM Fisher matrices (FP64 duals through the six modes, for FP64
    and mixed plans) against the oracle's dual-number Fisher."""
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    rng = np.random.default_rng(9)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(2)])
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision=precision, reference_frequency=1e-4,
                            approximant="IMRPhenomHM", cut_factor=1.2, max_batch=4)
    got = eng.fisher_matrix(thetas).cpu().numpy()
    want = oracle_plan(oracle, g, dets, cut_factor=1.2).fisher(thetas)
    s = np.sqrt(np.einsum("bii->bi", want))
    assert np.max(np.abs(got - want) / (s[:, :, None] * s[:, None, :])) < 1e-9
