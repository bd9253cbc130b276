"""IMRPhenomD waveform producer on CUDA (the waveform-container contract the
reference's likelihoods consume: interface_bilby.py:97, antenna.py:438-458,
interface_ripple.py:44-50).  t_c is fixed to zero inside the waveform; the
response applies it (interface_ripple.py:135-147).
"""

import math

import numpy as np
import torch

from .. import _lib

PARAM_NAMES = ("ln_chirp_mass", "mass_ratio", "chi_1", "chi_2", "ln_luminosity_distance", "cos_inclination",
               "ecliptic_longitude", "sin_ecliptic_latitude", "polarization", "reference_phase", "coalescence_time")


def q_from_eta(eta):
    """m1/m2 >= 1 from the symmetric mass ratio."""
    eta = min(float(eta), 0.25)
    return (1.0 - 2.0 * eta + math.sqrt(max(0.0, 1.0 - 4.0 * eta))) / (2.0 * eta)


def theta_from_parameters(p):
    """11-parameter vector from a reference-style parameter dict / namedtuple.

    Accepts (chirp_mass, symmetric_mass_ratio | mass_ratio | mass_1 & mass_2),
    chi_1, chi_2, luminosity_distance [Mpc], inclination, reference_phase and,
    when present, ecliptic_longitude, ecliptic_latitude, polarization,
    coalescence_time.
    """
    g = (lambda k, d=None: p.get(k, d)) if isinstance(p, dict) else (lambda k, d=None: getattr(p, k, d))
    if g("mass_1") is not None and g("mass_2") is not None and g("chirp_mass") is None:
        m1, m2 = float(g("mass_1")), float(g("mass_2"))
        q = max(m1, m2) / min(m1, m2)
        mc = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2
    else:
        mc = float(g("chirp_mass"))
        if g("mass_ratio") is not None:
            q = float(g("mass_ratio"))
            q = q if q >= 1.0 else 1.0 / q
        else:
            q = q_from_eta(g("symmetric_mass_ratio"))
    return np.array([
        math.log(mc), q, float(g("chi_1")), float(g("chi_2")), math.log(float(g("luminosity_distance"))),
        math.cos(float(g("inclination"))), float(g("ecliptic_longitude", 0.0)),
        math.sin(float(g("ecliptic_latitude", 0.0))), float(g("polarization", 0.0)), float(g("reference_phase")),
        float(g("coalescence_time", 0.0)),
    ], dtype=np.float64)


class IMRPhenomD:
    """(2,2)-mode IMRPhenomD polarisations and t(f) on a frequency grid."""

    required_params = ("chirp_mass", "symmetric_mass_ratio", "chi_1", "chi_2", "luminosity_distance",
                       "reference_phase", "inclination")

    def __init__(self, frequencies, reference_frequency, cutoff_frequency=math.inf):
        self.frequencies = torch.as_tensor(np.asarray(frequencies), dtype=torch.float64, device="cuda").contiguous()
        self.reference_frequency = float(reference_frequency)
        self.cutoff_frequency = float(cutoff_frequency)
        n = self.frequencies.numel()
        self.waveform_container = {
            "plus": torch.zeros(n, dtype=torch.complex128, device="cuda"),
            "cross": torch.zeros(n, dtype=torch.complex128, device="cuda"),
            "tf": torch.zeros(n, dtype=torch.float64, device="cuda"),
        }

    def _run(self, theta, out):
        theta = np.ascontiguousarray(theta, dtype=np.float64).copy()
        theta[10] = 0.0  # t_c is applied by the response
        n = self.frequencies.numel()
        _lib.check(_lib.load().pes_phenomd(
            _lib.ptr(theta), _lib.ptr(self.frequencies), n, self.reference_frequency,
            min(self.cutoff_frequency, 1e300), _lib.ptr(out["plus"]), _lib.ptr(out["cross"]), _lib.ptr(out["tf"]),
            _lib.stream_handle()))
        return out

    def update_waveform(self, parameters):
        """tiwave-style: fill ``waveform_container`` in place."""
        self._run(theta_from_parameters(parameters), self.waveform_container)

    def get_waveform(self, params):
        """ripple-style: return a fresh ``{"plus", "cross", "tf"}`` dict."""
        n = self.frequencies.numel()
        out = {"plus": torch.empty(n, dtype=torch.complex128, device="cuda"),
               "cross": torch.empty(n, dtype=torch.complex128, device="cuda"),
               "tf": torch.empty(n, dtype=torch.float64, device="cuda")}
        return self._run(theta_from_parameters(params), out)

    def from_theta(self, theta):
        n = self.frequencies.numel()
        out = {"plus": torch.empty(n, dtype=torch.complex128, device="cuda"),
               "cross": torch.empty(n, dtype=torch.complex128, device="cuda"),
               "tf": torch.empty(n, dtype=torch.float64, device="cuda")}
        return self._run(theta, out)

    __call__ = get_waveform
