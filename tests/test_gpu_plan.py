"""Batched FP64 plan (pes_lnl_batch / pes_lnl_grad_batch) against the oracle.

Bars (spec parity for the plain FP64 path): |dlnL| <= 1e-6 absolute,
dense A/E/T model within 1e-10 of the per-bin response magnitude, gradient
within 1e-7 relative of the oracle's forward-mode dual numbers.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, make_dataset, perturbed, random_prior_theta  # noqa: E402

DUR, DT, FMIN, FMAX = 2.0 ** 18, 8.0, 1e-4, 0.03


def lisa(oracle, gen="1.5"):
    return ("lisa", oracle.heliocentric(2.5e9, 0.0, -np.pi / 9), gen, oracle.PSD_PRESETS["LISA_SciRDv1"])


def tianqin(oracle, gen="1.5"):
    return ("tianqin", oracle.geocentric(np.sqrt(3.0) * 1e8), gen,
            dict(oms_level=1e-24, acc_level=1e-30, arm_length_sec=np.sqrt(3) * 1e8 / oracle.C_SI, tianqin=True))


def cuda_detectors(g, dets, grid=None):
    from pespace_gb300.detector.antenna import FDResponseModelMarset2018, InterferometerAntenna
    from pespace_gb300.detector.orbit import KaplerianHeliocentric, KeplerianGeocentric
    from pespace_gb300.detector.tdi import FDMichelsonConstantEqualArm, TDIChannelData

    out = []
    for name, orb_desc, gen, data, psd in dets:
        td = TDIChannelData()
        dur, dt, fmin, fmax = grid if grid is not None else (DUR, DT, FMIN, FMAX)
        td.set_fd_data_from_zero(("A", "E", "T"), dur, dt, 0.0, fmin, fmax)
        td.fd_data.copy_(torch.as_tensor(data, device="cuda"))
        td.fd_noise_power_density = torch.as_tensor(psd, device="cuda")
        if orb_desc.kind == 0:
            orb = KaplerianHeliocentric(orb_desc.arm_sec * 299792458.0, orb_desc.rotation_initial,
                                        orb_desc.revolution_initial)
        else:
            orb = KeplerianGeocentric(orb_desc.arm_sec * 299792458.0, orb_desc.rotation_initial,
                                      orb_desc.revolution_initial)
        out.append(InterferometerAntenna(name, td, orb, FDResponseModelMarset2018(),
                                         FDMichelsonConstantEqualArm(gen, True)))
    return tuple(out)


@pytest.fixture(scope="module")
def dataset(oracle):
    tc = DUR - 20000.0
    th0 = config0_theta(tc)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle), tianqin(oracle)], th0)
    return g, dets, th0


def test_lnl_injection_and_perturbed(cuda_lib, oracle, dataset):
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    rng = np.random.default_rng(11)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(7)])
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="fp64", reference_frequency=1e-4, max_batch=16)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4)
    want = plan.lnl(thetas)
    assert np.all(eng.last_status.cpu().numpy() == 0)
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-6)
    # determinism: bitwise identical on repeat
    again = eng.log_likelihood_batch(thetas).cpu().numpy()
    assert np.array_equal(got, again)


def test_dense_model_parity(cuda_lib, oracle, dataset):
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision="fp64", reference_frequency=1e-4, max_batch=4)
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4)
    for d in range(2):
        for orth in (True, False):
            got = eng.model_tdi(th0, det=d, orthogonal=orth).cpu().numpy()
            want = plan.model_tdi(d, th0, orthogonal=orth)
            mag = np.sqrt(np.sum(np.abs(want) ** 2, axis=0)) + 1e-300
            live = mag > 1e-300
            assert np.max(np.abs(got - want)[:, live] / mag[live]) < 1e-10


def test_network_subset_and_generation(cuda_lib, oracle):
    from pespace_gb300.inference import WhittleLikelihood

    tc = DUR - 30000.0
    th0 = config0_theta(tc)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle, "2.0"), tianqin(oracle, "2.0")], th0, seed=5)
    rng = np.random.default_rng(3)
    thetas = np.stack([th0] + [perturbed(th0, rng, 3.0) for _ in range(5)])
    for chans in (("A", "E", "T"), ("A", "E"), ("T",)):
        eng = WhittleLikelihood(cuda_detectors(g, dets), channels=chans, precision="fp64", reference_frequency=1e-4,
                                max_batch=8)
        got = eng.log_likelihood_batch(thetas).cpu().numpy()
        plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, channels=chans)
        np.testing.assert_allclose(got, plan.lnl(thetas), rtol=1e-11, atol=1e-6)


def test_prior_batch_with_cutoff(cuda_lib, oracle, dataset):
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    rng = np.random.default_rng(2026)
    thetas = random_prior_theta(rng, 24, th0[10])
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="fp64", reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=32)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4, cut_factor=1.2)
    np.testing.assert_allclose(got, plan.lnl(thetas, nthreads=8), rtol=1e-11, atol=1e-6)


def test_gradient_vs_oracle_duals(cuda_lib, oracle, dataset):
    from pespace_gb300.inference import WhittleLikelihood, log_likelihood

    g, dets, th0 = dataset
    rng = np.random.default_rng(5)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision="fp64", reference_frequency=1e-4, max_batch=8)
    lnl, grad = eng.log_likelihood_and_grad(thetas)
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4)
    w_lnl, w_grad = plan.lnl(thetas, grad=True, nthreads=8)
    np.testing.assert_allclose(lnl.cpu().numpy(), w_lnl, rtol=1e-11, atol=1e-6)
    gg = grad.cpu().numpy()
    scale = np.abs(w_grad) + 1e-9 * np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(gg - w_grad) / scale) < 1e-7
    # torch.autograd route
    t = torch.as_tensor(thetas, device="cuda").requires_grad_(True)
    log_likelihood(t, eng).sum().backward()
    np.testing.assert_allclose(t.grad.cpu().numpy(), gg, rtol=0, atol=0)


def test_edge_cases_and_status(cuda_lib, oracle, dataset):
    from pespace_gb300 import _lib
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="fp64", reference_frequency=1e-4, max_batch=4)
    bad = np.stack([th0, th0, th0, th0])
    bad[1, 1] = 0.5      # q < 1
    bad[2, 2] = 1.0      # |chi1| = 1
    bad[3, 6] = np.nan   # NaN sky
    lnl = eng.log_likelihood_batch(bad).cpu().numpy()
    st = eng.last_status.cpu().numpy()
    assert st[0] == 0 and np.isfinite(lnl[0])
    assert list(st[1:]) == [2, 2, 2] and np.all(np.isneginf(lnl[1:]))
    # empty batch and an oversized one
    assert eng.log_likelihood_batch(np.zeros((0, 11))).numel() == 0
    lib = _lib.load()
    th = torch.as_tensor(np.stack([th0] * 5), device="cuda")
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    assert lib.pes_lnl_batch(eng._plan, _lib.ptr(th), 5, _lib.ptr(out), None, None) == _lib.PES_EINVAL


def test_gradient_central_differences(cuda_lib, oracle, dataset):
    """FP64 plan gradient against central finite differences of its own lnL
    (step 1e-6 relative: 1e-6 in ln Mc and ln D_L, 1e-6 max(|x|, 1) for the
    others).  The mixed
    plan's lnL carries FP32 rounding of ~1e-9 |lnL|, which such a step turns
    into differences far above its gradient error; its gradient is checked
    against the oracle's dual numbers instead."""
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="fp64", reference_frequency=1e-4, max_batch=32)
    rng = np.random.default_rng(17)
    base = np.stack([th0, perturbed(th0, rng)])
    _, grad = eng.log_likelihood_and_grad(base)
    grad = grad.cpu().numpy()
    for b in range(base.shape[0]):
        steps = 1e-6 * np.maximum(np.abs(base[b]), 1.0)
        steps[[0, 4]] = 1e-6  # ln Mc, ln D_L: a relative step of 1e-6 in Mc and D_L
        pts = np.repeat(base[b][None], 22, axis=0)
        for k in range(11):
            pts[2 * k, k] += steps[k]
            pts[2 * k + 1, k] -= steps[k]
        v = eng.log_likelihood_batch(pts).cpu().numpy()
        fd = (v[0::2] - v[1::2]) / (2 * steps)
        norm = np.linalg.norm(grad[b])
        assert np.max(np.abs(fd - grad[b])) / norm < 1e-4, (b, fd, grad[b])


def test_reference_parameter_tuple_calls(cuda_lib, oracle, dataset):
    """likelihood_param_type / log_likelihood(namedtuple) as a JAX-style sampler
    calls them: scalar fields give a float, array fields a batched tensor."""
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="fp64", reference_frequency=1e-4, max_batch=8)
    rng = np.random.default_rng(29)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    eta = thetas[:, 1] / (1 + thetas[:, 1]) ** 2
    P = eng.likelihood_param_type
    assert P._fields[-4:] == ("ecliptic_longitude", "ecliptic_latitude", "polarization", "coalescence_time")
    batch = P(chirp_mass=np.exp(thetas[:, 0]), symmetric_mass_ratio=eta, chi_1=thetas[:, 2], chi_2=thetas[:, 3],
              luminosity_distance=np.exp(thetas[:, 4]), reference_phase=thetas[:, 9],
              inclination=np.arccos(thetas[:, 5]), ecliptic_longitude=thetas[:, 6],
              ecliptic_latitude=np.arcsin(thetas[:, 7]), polarization=thetas[:, 8], coalescence_time=thetas[:, 10])
    want = eng.log_likelihood_batch(thetas).cpu().numpy()
    got = eng.log_likelihood(batch).cpu().numpy()
    assert np.allclose(got, want, rtol=1e-12, atol=1e-9)
    one = eng.log_likelihood(P(*[np.asarray(f)[0] for f in batch]))
    assert isinstance(one, float) and abs(one - want[0]) <= 1e-9 + 1e-12 * abs(want[0])


def test_reference_constructor_signature(cuda_lib, oracle, dataset):
    """WhittleLikelihoodCuda(waveform, detector, channels), the reference's
    WhittleLikelihoodJax constructor: the same plan as WhittleLikelihood with
    the waveform's reference frequency, and the reference's argument checks."""
    from pespace_gb300.inference import WhittleLikelihood, WhittleLikelihoodCuda
    from pespace_gb300.waveform import IMRPhenomD

    g, dets, th0 = dataset
    cdets = cuda_detectors(g, dets[:1])
    freqs = cdets[0].tdi_data.data_info.frequency_samples_array
    like = WhittleLikelihoodCuda(IMRPhenomD(freqs, 1e-4), cdets, ("A", "E", "T"), max_batch=8)
    ref = WhittleLikelihood(cdets, precision="fp64", reference_frequency=1e-4, max_batch=8)
    rng = np.random.default_rng(31)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    assert torch.equal(like.log_likelihood_batch(thetas), ref.log_likelihood_batch(thetas))
    assert like.likelihood_param_type._fields == ref.likelihood_param_type._fields
    with pytest.raises(ValueError):
        WhittleLikelihoodCuda(IMRPhenomD(freqs[:-1], 1e-4), cdets, ("A", "E", "T"))
    with pytest.raises(ValueError):
        WhittleLikelihoodCuda(IMRPhenomD(freqs, 1e-4), cdets, ("A", "X"))


def test_optimal_snr(cuda_lib, oracle, dataset):
    """InterferometerAntenna.get_optimal_snr: rho_c^2 = 4 df sum |h_c|^2 / S_c
    of the plugin response, against the oracle's A/E/T model."""
    from pespace_gb300.waveform import IMRPhenomD

    g, dets, th0 = dataset
    det = cuda_detectors(g, dets[:1])[0]
    wf = IMRPhenomD(det.tdi_data.data_info.frequency_samples_array, 1e-4)
    snr = det.get_optimal_snr(wf.from_theta(th0), th0[6], np.arcsin(th0[7]), th0[8], th0[10])
    h = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4).model_tdi(0, th0)
    S = np.asarray(dets[0][4])
    w = np.where(S > 0, 1.0 / np.where(S > 0, S, 1.0), 0.0)
    want = 4.0 * g["df"] * np.sum(np.abs(h) ** 2 * w, axis=1)
    for k, c in enumerate("AET"):
        assert abs(snr[c] ** 2 - want[k]) <= 1e-8 * want.sum(), c
    assert abs(snr["total"] ** 2 - want.sum()) <= 1e-8 * want.sum()
    assert snr["total"] > 0
