"""Parity at the benchmark grid: T = 2^22 s, dt = 8 s, 1e-4..0.03 Hz (125 410
bins), LISA-like detector, TDI 1.5, where 2 pi f t_c reaches ~8e5 rad.

* FP64 plan against the oracle: the dense A/E/T model per bin within 1e-10 of
  the per-bin response scale, lnL at the injection and at 32 prior draws
  (cut at 1.2 f_RD) within 1e-6 (absolute; 1e-11 relative for the loud ones).
* Mixed plan against the oracle on the same 32 draws and the injection:
  |dlnL| <= 1e-2 for every sample.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, make_dataset  # noqa: E402
from tests.test_gpu_plan import cuda_detectors, lisa  # noqa: E402

GRID = (2.0 ** 22, 8.0, 1e-4, 0.03)


@pytest.fixture(scope="module")
def bench_grid(oracle):
    th0 = config0_theta(GRID[0] - 86400.0)
    g, dets = make_dataset(oracle, *GRID, [lisa(oracle)], th0, seed=2026)
    from pespace_gb300.workloads import prior_samples

    thetas = np.concatenate([th0[None], prior_samples(np.random.default_rng(2026), 32, th0[10])])
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2)
    want = plan.lnl(thetas, nthreads=16)
    return g, dets, th0, thetas, want


def test_bench_grid_fp64_model(cuda_lib, oracle, bench_grid):
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0, _, _ = bench_grid
    eng = WhittleLikelihood(cuda_detectors(g, dets, GRID), precision="fp64", reference_frequency=1e-4, max_batch=2)
    assert int(eng.desc.nbins) == 125410
    got = eng.model_tdi(th0).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4).model_tdi(0, th0)
    mag = np.sqrt(np.sum(np.abs(want) ** 2, axis=0))
    live = mag > 0
    assert np.max(np.abs(got - want)[:, live] / mag[live]) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bench_grid_prior_draws(cuda_lib, oracle, bench_grid, precision):
    from pespace_gb300.inference import WhittleLikelihood

    g, dets, th0, thetas, want = bench_grid
    eng = WhittleLikelihood(cuda_detectors(g, dets, GRID), precision=precision, reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=40)
    got = eng.log_likelihood_batch(thetas).cpu().numpy()
    assert np.all(eng.last_status.cpu().numpy() == 0)
    err = np.abs(got - want)
    if precision == "fp64":
        assert np.all(err <= 1e-6 + 1e-11 * np.abs(want)), np.sort(err)[-4:]
    else:
        assert np.all(err <= 1e-2), np.sort(err)[-4:]
