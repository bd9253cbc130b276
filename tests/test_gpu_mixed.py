"""Mixed-precision plan (FP64 sparse grid + FP32 dense bulk) against the FP64 oracle.

Bar: |dlnL| <= 1e-2 against the FP64 oracle, for every sample.  The plan
adds the splines' midpoint error back per bin and re-evaluates the dense
range of the samples whose estimated FP32 rounding or remaining spline error
could reach the bar (templates far louder than the data): in float-float from
the same splines, or exactly where the spline estimate alone is too large.  Light
systems whose lowest bins lie decades before coalescence go through the exact
FP64 bins of the mixed plan.  The gradient is the exact gradient of the
interpolated model, checked against the oracle's forward-mode duals to 1e-3
of the gradient norm.
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


def engines(g, dets, n_sparse=1024, **kw):
    from pespace_gb300.inference import WhittleLikelihood

    return (WhittleLikelihood(cuda_detectors(g, dets), precision="mixed", reference_frequency=1e-4, n_sparse=n_sparse,
                              **kw),
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
    assert err[0] <= 1e-2  # the injection
    assert np.all(err <= 1e-2), err
    # deterministic forward
    assert np.array_equal(got, mixed.log_likelihood_batch(thetas).cpu().numpy())


def taiji(oracle, gen="1.5"):
    return ("taiji", oracle.heliocentric(3.0e9, 0.0, np.pi / 9), gen,
            dict(oms_level=(8e-12) ** 2, acc_level=(3e-15) ** 2, arm_length_sec=3.0e9 / oracle.C_SI))


@pytest.mark.parametrize("network", [False, True])
def test_mixed_prior_batch_cutoff(cuda_lib, oracle, network):
    tc = DUR - 20000.0
    th0 = config0_theta(tc)
    dl = [lisa(oracle), taiji(oracle)] if network else [lisa(oracle)]
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, dl, th0, seed=7)
    rng = np.random.default_rng(2026)
    thetas = random_prior_theta(rng, 48, th0[10])
    mixed, _ = engines(g, dets, max_batch=64, cut_factor=1.2)
    got = mixed.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(thetas, nthreads=8)
    err = np.abs(got - want)
    assert np.all(err <= 1e-2), np.sort(err)[-5:]


@pytest.mark.parametrize("network", [False, True])
def test_mixed_float_float_refinement(cuda_lib, oracle, network):
    """Every sample's dense range re-evaluated (the paths the samples whose
    error estimates approach the target take: float-float from the splines,
    exact where the splines' estimate alone is too large): within 1e-2 of the
    oracle for every sample, the same lnL from the lnL and lnL+gradient calls,
    and the work report counts them all."""
    tc = DUR - 20000.0
    th0 = config0_theta(tc)
    dl = [lisa(oracle), taiji(oracle)] if network else [lisa(oracle)]
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, dl, th0, seed=7)
    rng = np.random.default_rng(2026)
    thetas = np.concatenate([th0[None], random_prior_theta(rng, 31, th0[10])])
    mixed, _ = engines(g, dets, max_batch=32, cut_factor=1.2)
    assert not mixed.refine_all
    default = mixed.log_likelihood_batch(thetas).cpu().numpy()
    mixed.refine_all = True
    assert mixed.refine_all
    lnl, _ = mixed.log_likelihood_and_grad(thetas)
    got = mixed.log_likelihood_batch(thetas)
    assert torch.equal(lnl, got)
    work = mixed.last_work(32)
    assert work["refined_ff"] + work["refined_exact"] == work["samples"] == 32
    assert work["refined_ff"] >= 16
    got = got.cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(thetas, nthreads=8)
    err = np.abs(got - want)
    assert np.all(err <= 1e-2), np.sort(err)[-5:]
    assert np.median(err) <= np.median(np.abs(default - want)) + 1e-6
    mixed.refine_all = False
    assert np.array_equal(mixed.log_likelihood_batch(thetas).cpu().numpy(), default)


def test_mixed_taiji_t_channel_zero(cuda_lib, oracle):
    """Taiji (L = 10 s) on a band reaching 0.1 Hz holds the T channel's zero
    f = 1/L = 0.0999 Hz, where T's transfer and its PSD vanish together and
    1/S_T grows as (f - 1/L)^-4.  The mixed plan evaluates the bins about it
    exactly: sources whose ringdown reaches it within 1e-2 of the oracle
    (lnL, also with every sample refined) and within 1e-3 of the gradient
    norm; the window bins are reported as exact bins."""
    dur, dt = 2.0 ** 18, 4.0
    th0 = config0_theta(dur - 20000.0)
    th0[0] -= np.log(10.0)  # total mass 1.5e5 Msun: f_RD near 0.1 Hz
    g, dets = make_dataset(oracle, dur, dt, 1e-4, 0.1, [taiji(oracle)], th0, seed=3)
    rng = np.random.default_rng(19)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(7)])
    from pespace_gb300.inference import WhittleLikelihood

    mixed = WhittleLikelihood(cuda_detectors(g, dets, grid=(dur, dt, 1e-4, 0.1)), precision="mixed",
                              reference_frequency=1e-4, max_batch=8)
    lnl, grad = mixed.log_likelihood_and_grad(thetas)
    work = mixed.last_work(8)
    kcut = int(np.searchsorted(g["freqs"], 0.1, side="right"))
    assert work["fp64_bins"] >= 8 * 64 and work["dense_bins"] + work["fp64_bins"] <= 8 * kcut
    w_lnl, w_grad = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4).lnl(
        thetas, grad=True, nthreads=8)
    err = np.abs(lnl.cpu().numpy() - w_lnl)
    assert np.all(err <= 1e-2), err
    norm = np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(grad.cpu().numpy() - w_grad) / norm) < 1e-3
    mixed.refine_all = True
    err = np.abs(mixed.log_likelihood_batch(thetas).cpu().numpy() - w_lnl)
    assert np.all(err <= 1e-2), err


def test_mixed_geocentric_network(cuda_lib, oracle, dataset):
    """LISA + TianQin: the geocentric constellation's 3.65-day rotation makes
    most inspiral bins exact (FP64); lnL and gradient against the oracle."""
    g, dets, th0 = dataset
    rng = np.random.default_rng(31)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)] + list(random_prior_theta(rng, 4, th0[10])))
    mixed, _ = engines(g, dets, max_batch=8, cut_factor=1.2)
    lnl, grad = mixed.log_likelihood_and_grad(thetas)
    w_lnl, w_grad = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(
        thetas, grad=True, nthreads=8)
    err = np.abs(lnl.cpu().numpy() - w_lnl)
    assert np.all(err <= 1e-2), err
    norm = np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(grad.cpu().numpy() - w_grad) / norm) < 1e-3


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


def test_mixed_dense_staging_variants(cuda_lib, oracle, dataset, monkeypatch):
    """The gradient pass of the dense stage with its run inputs copied one run
    ahead into shared memory (cp.async) and with plain loads: the same lnL bit
    for bit and the same gradient up to the order of the FP32 moment atomics
    (LISA + TianQin, so exact runs are skipped in both)."""
    g, dets, th0 = dataset
    rng = np.random.default_rng(41)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(2)] + list(random_prior_theta(rng, 3, th0[10])))
    monkeypatch.setenv("PES_DENSE_STAGE", "1")
    staged, _ = engines(g, dets, max_batch=8, cut_factor=1.2)
    monkeypatch.setenv("PES_DENSE_STAGE", "0")
    plain, _ = engines(g, dets, max_batch=8, cut_factor=1.2)
    l1, g1 = staged.log_likelihood_and_grad(thetas)
    l0, g0 = plain.log_likelihood_and_grad(thetas)
    assert torch.equal(l1, l0)
    assert torch.equal(staged.log_likelihood_batch(thetas), l0)
    norm = torch.linalg.norm(g0, dim=1, keepdim=True)
    assert torch.max(torch.abs(g1 - g0) / norm).item() < 1e-5


@pytest.mark.parametrize("n_sparse", [600, 2048, 3000])
def test_mixed_other_grids(cuda_lib, oracle, dataset, n_sparse):
    """Non-default sparse grids: 600 nodes (register segments of 19 rows),
    2048 nodes (register segments of 64 rows) and 3000 nodes (the
    global-scratch spline kernels)."""
    g, dets, th0 = dataset
    rng = np.random.default_rng(3)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    mixed, _ = engines(g, dets[:1], n_sparse=n_sparse, max_batch=4)
    lnl, grad = mixed.log_likelihood_and_grad(thetas)
    w_lnl, w_grad = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4).lnl(
        thetas, grad=True, nthreads=8)
    err = np.abs(lnl.cpu().numpy() - w_lnl)
    tol = 1e-2 if n_sparse >= 1024 else 5e-2  # spline error grows as (node spacing)^4
    assert np.all(err <= tol), err
    norm = np.linalg.norm(w_grad, axis=1, keepdims=True)
    assert np.max(np.abs(grad.cpu().numpy() - w_grad) / norm) < 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_cuda_graph_replay(cuda_lib, oracle, dataset, precision):
    """A captured lnL+gradient call replays identically to the direct call,
    on new parameters too (mixed gradients within FP32 atomic-order noise)."""
    from pespace_gb300.inference import CapturedStep, WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision=precision, reference_frequency=1e-4,
                            max_batch=8)
    rng = np.random.default_rng(23)
    step = CapturedStep(eng, 8)
    for _ in range(2):
        thetas = np.stack([perturbed(th0, rng) for _ in range(8)])
        lnl, grad = step(thetas)
        lnl, grad = lnl.clone(), grad.clone()
        want_lnl, want_grad = eng.log_likelihood_and_grad(thetas)
        assert torch.equal(lnl, want_lnl)
        if precision == "fp64":
            assert torch.equal(grad, want_grad)
        else:
            assert torch.allclose(grad, want_grad, rtol=1e-5, atol=1e-6 * float(want_grad.abs().max()))


def test_mixed_tdi2_prefactor_zero(cuda_lib, oracle):
    """TDI 2.0 up to 0.1 Hz: the generation prefactor (1 - D^2)(1 - D^4) has a
    double zero at f L = 1/2 (0.06 Hz), where the PSD vanishes too.  The mixed
    plan keeps that factor out of its splines and applies it per bin (with the
    factor inside the splines the errors near 0.06 Hz reached |dlnL| ~ 100).
    Every sample within 1e-2 of the oracle."""
    from pespace_gb300.inference import WhittleLikelihood

    grid = (2.0 ** 16, 5.0, 1e-4, 0.1)
    th0 = config0_theta(grid[0] - 8000.0)
    g, dets = make_dataset(oracle, *grid, [lisa(oracle, "2.0")], th0, seed=12)
    rng = np.random.default_rng(77)
    thetas = np.concatenate([th0[None], random_prior_theta(rng, 31, th0[10])])
    eng = WhittleLikelihood(cuda_detectors(g, dets, grid), precision="mixed", reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=32)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(thetas, nthreads=8)
    err = np.abs(got - want)
    assert np.all(err <= 1e-2), np.sort(err)[-5:]


def test_mixed_edge_cases_and_status(cuda_lib, oracle, dataset):
    """Out-of-domain and NaN samples in a mixed batch: status 2 and lnL = -inf,
    zero gradient rows, the valid neighbours unaffected; an empty batch; a batch
    beyond max_batch through the C ABI is rejected; channel subsets."""
    from pespace_gb300 import _lib
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0 = dataset
    eng = WhittleLikelihood(cuda_detectors(g, dets[:1]), precision="mixed", reference_frequency=1e-4, max_batch=4)
    bad = np.stack([th0, th0, th0, th0])
    bad[1, 1] = 0.5      # q < 1
    bad[2, 3] = -1.0     # |chi2| = 1
    bad[3, 10] = np.nan  # NaN t_c
    lnl, grad = eng.log_likelihood_and_grad(bad)
    lnl, grad, st = lnl.cpu().numpy(), grad.cpu().numpy(), eng.last_status.cpu().numpy()
    assert st[0] == 0 and np.isfinite(lnl[0]) and np.all(np.isfinite(grad[0]))
    assert list(st[1:]) == [2, 2, 2] and np.all(np.isneginf(lnl[1:])) and np.all(grad[1:] == 0)
    alone = eng.log_likelihood_batch(th0[None]).cpu().numpy()
    assert lnl[0] == alone[0]
    assert eng.log_likelihood_batch(np.zeros((0, 11))).numel() == 0
    lib = _lib.load()
    th = torch.as_tensor(np.stack([th0] * 5), device="cuda")
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    assert lib.pes_lnl_batch(eng._plan, _lib.ptr(th), 5, _lib.ptr(out), None, None) == _lib.PES_EINVAL
    # channel subsets against the oracle
    rng = np.random.default_rng(41)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    for chans in (("A", "E"), ("T",)):
        sub = WhittleLikelihood(cuda_detectors(g, dets[:1]), channels=chans, precision="mixed",
                                reference_frequency=1e-4, max_batch=4)
        got = sub.log_likelihood_batch(thetas).cpu().numpy()
        plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4, channels=chans)
        want = plan.lnl(thetas)
        assert np.all(np.abs(got - want) <= 1e-2), (chans, got - want)


def test_launch_options_and_autotune(cuda_lib, oracle, dataset):
    """Launch options change speed only: every staging choice and per-sample
    block size gives the same lnL bit for bit (gradient up to the order of
    the FP32 moment atomics); the autotuner keeps one of its candidates."""
    from pespace_gb300.inference.autotune import CANDIDATES, set_option

    g, dets, th0 = dataset
    rng = np.random.default_rng(43)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(2)] + list(random_prior_theta(rng, 3, th0[10])))
    mixed, fp64 = engines(g, dets, max_batch=8, cut_factor=1.2)
    assert mixed.launch_options == {"dense_stage": 0, "sample_threads": 8}  # small inputs: direct loads
    l0, g0 = mixed.log_likelihood_and_grad(thetas)
    norm = torch.linalg.norm(g0, dim=1, keepdim=True)
    for stage in CANDIDATES["dense_stage"]:
        for threads in CANDIDATES["sample_threads"] + (1, 128):
            set_option(mixed, "dense_stage", stage)
            set_option(mixed, "sample_threads", threads)
            l1, g1 = mixed.log_likelihood_and_grad(thetas)
            assert torch.equal(l1, l0), (stage, threads)
            assert torch.equal(mixed.log_likelihood_batch(thetas), l0), (stage, threads)
            assert torch.max(torch.abs(g1 - g0) / norm).item() < 1e-5, (stage, threads)
    report = mixed.autotune(thetas, reps=2)
    assert set(report) == {"dense_stage", "sample_threads"}
    assert mixed.launch_options == {k: v["chosen"] for k, v in report.items()}
    assert all(v["chosen"] in CANDIDATES[k] and v["ms"][v["chosen"]] > 0 for k, v in report.items())
    assert torch.equal(mixed.log_likelihood_batch(thetas), l0)
    # FP64 plans: only the per-sample block size
    w0 = fp64.log_likelihood_batch(thetas)
    report = fp64.autotune(thetas, grad=False, reps=1)
    assert set(report) == {"sample_threads"} and fp64.launch_options["dense_stage"] == 0
    assert torch.equal(fp64.log_likelihood_batch(thetas), w0)
