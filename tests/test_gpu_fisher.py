"""pes_fisher_batch against the oracle's FP64 dual-number Fisher matrices."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, make_dataset, perturbed  # noqa: E402
from tests.test_gpu_mixed import taiji  # noqa: E402
from tests.test_gpu_plan import DT, DUR, FMAX, FMIN, cuda_detectors, lisa  # noqa: E402


def _normalised_err(got, want):
    s = np.sqrt(np.einsum("bii->bi", want))
    scale = s[:, :, None] * s[:, None, :]
    return np.max(np.abs(got - want) / scale)


@pytest.mark.parametrize("network", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fisher_vs_oracle(cuda_lib, oracle, network, precision):
    from pespace_gb300.inference import WhittleLikelihood

    th0 = config0_theta(DUR - 20000.0)
    dl = [lisa(oracle), taiji(oracle)] if network else [lisa(oracle)]
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, dl, th0, seed=4)
    rng = np.random.default_rng(8)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(2)])
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision=precision, reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=4)
    got = eng.fisher_matrix(thetas).cpu().numpy()
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).fisher(thetas)
    assert np.all(eng.last_status.cpu().numpy() == 0)
    assert np.array_equal(got, np.swapaxes(got, 1, 2))
    # FP64 plans: FP64 duals through the model; mixed plans: FP32 structured
    # derivatives (the bar of the 11x11 Fisher rows is 1e-4 relative)
    assert _normalised_err(got, want) < (1e-9 if precision == "fp64" else 1e-5)
    # deterministic
    assert np.array_equal(got, eng.fisher_matrix(thetas).cpu().numpy())


def test_fisher_reference_call_and_domain(cuda_lib, oracle):
    from pespace_gb300.inference import WhittleLikelihood, fisher_matrix

    th0 = config0_theta(DUR - 20000.0)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle)], th0, seed=4)
    eng = WhittleLikelihood(cuda_detectors(g, dets), precision="fp64", reference_frequency=1e-4, max_batch=2)
    single = fisher_matrix(eng, th0)
    assert single.shape == (11, 11)
    bad = th0.copy()
    bad[1] = 0.5  # q < 1 is outside the domain
    batch = fisher_matrix(eng, np.stack([th0, bad, th0]), batch_size=2)
    assert batch.shape == (3, 11, 11)
    assert torch.equal(batch[0], single) and torch.equal(batch[2], single)
    assert torch.isnan(batch[1]).all()
    params = dict(chirp_mass=float(np.exp(th0[0])), mass_ratio=float(th0[1]), chi_1=th0[2], chi_2=th0[3],
                  luminosity_distance=float(np.exp(th0[4])), inclination=float(np.arccos(th0[5])),
                  ecliptic_longitude=th0[6], ecliptic_latitude=float(np.arcsin(th0[7])), polarization=th0[8],
                  reference_phase=th0[9], coalescence_time=th0[10])
    from_dict = fisher_matrix(eng, params).cpu().numpy()
    assert _normalised_err(from_dict[None], single.cpu().numpy()[None]) < 1e-12
