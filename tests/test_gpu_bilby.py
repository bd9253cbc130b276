"""LikelihoodBilbyInterface.log_likelihood (interface_bilby.py:78-116) on a
two-detector network (LISA-like heliocentric + TianQin-like geocentric): the
waveform object fills its container from the parameter dict, each detector
updates its response and the per-detector Whittle sums are added.  Against
the oracle's lnL of the same data and the batched FP64 plan, for IMRPhenomD
and the six-mode IMRPhenomHM container."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tests.helpers import config0_theta, perturbed  # noqa: E402
from tests.test_gpu_plan import cuda_detectors, dataset  # noqa: E402,F401


def _params(th):
    return {"chirp_mass": math.exp(th[0]), "mass_ratio": th[1], "chi_1": th[2], "chi_2": th[3],
            "luminosity_distance": math.exp(th[4]), "inclination": math.acos(th[5]),
            "ecliptic_longitude": th[6], "ecliptic_latitude": math.asin(th[7]), "polarization": th[8],
            "reference_phase": th[9], "coalescence_time": th[10]}


@pytest.mark.parametrize("approximant", ["IMRPhenomD", "IMRPhenomHM"])
def test_bilby_interface_network(cuda_lib, oracle, dataset, approximant):  # noqa: F811
    from pespace_gb300.inference import LikelihoodBilbyInterface, WhittleLikelihood
    from pespace_gb300.waveform import IMRPhenomD, IMRPhenomHM

    g, dets, th0 = dataset
    cdets = cuda_detectors(g, dets)
    freqs = cdets[0].tdi_data.frequency_samples.cpu().numpy()
    wf = (IMRPhenomD if approximant == "IMRPhenomD" else IMRPhenomHM)(freqs, 1e-4)
    like = LikelihoodBilbyInterface(wf, cdets, ("A", "E", "T"))
    rng = np.random.default_rng(19)
    thetas = np.stack([th0] + [perturbed(th0, rng) for _ in range(3)])
    got = []
    for th in thetas:
        like.parameters = _params(th)
        got.append(like.log_likelihood())
    got = np.array(got)
    # the reference's theta conversion is lossy only through acos/asin/exp round trips
    back = np.stack([np.array([math.log(math.exp(t[0])), t[1], t[2], t[3], math.log(math.exp(t[4])),
                               math.cos(math.acos(t[5])), t[6], math.sin(math.asin(t[7])), t[8], t[9], t[10]])
                     for t in thetas])
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, approximant=approximant).lnl(back)
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-6)
    plan = WhittleLikelihood(cdets, precision="fp64", reference_frequency=1e-4, approximant=approximant, max_batch=4)
    np.testing.assert_allclose(got, plan.log_likelihood_batch(back).cpu().numpy(), rtol=1e-11, atol=1e-6)
    # the per-detector sums: one detector alone is that detector's term
    single = LikelihoodBilbyInterface(wf, cdets[0], ("A", "E", "T"))
    one = single.log_likelihood(_params(thetas[0]))
    want1 = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets[:1]], 1e-4, approximant=approximant).lnl(
        back[:1])
    np.testing.assert_allclose(one, want1[0], rtol=1e-11, atol=1e-6)
