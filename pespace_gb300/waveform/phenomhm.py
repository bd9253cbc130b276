"""IMRPhenomHM waveform producer on CUDA: the mode-keyed waveform container
of the reference's higher-mode producers (pespace/waveform/interface_ripple.py:
155-235, {mode: {"plus", "cross", "tf"}}), consumed mode by mode by the
response (antenna.py:446-458), with IMRPhenomHM (London et al. 2018) in
place of the absent IMRPhenomXHM.  t_c is fixed to zero inside the waveform;
the response applies it (interface_ripple.py:135-147).
"""

import math

import numpy as np
import torch

from .. import _lib
from .phenomd import theta_from_parameters

MODES = ("22", "21", "33", "32", "44", "43")


class IMRPhenomHM:
    """Six-mode IMRPhenomHM: modes (2,2), (2,1), (3,3), (3,2), (4,4), (4,3)."""

    required_params = ("chirp_mass", "symmetric_mass_ratio", "chi_1", "chi_2", "luminosity_distance",
                       "reference_phase", "inclination")
    modes = MODES

    def __init__(self, frequencies, reference_frequency, cutoff_frequency=math.inf):
        self.frequencies = torch.as_tensor(np.asarray(frequencies), dtype=torch.float64, device="cuda").contiguous()
        self.reference_frequency = float(reference_frequency)
        self.cutoff_frequency = float(cutoff_frequency)
        self.waveform_container = self._empty()

    def _empty(self):
        n = self.frequencies.numel()
        hp = torch.zeros((len(MODES), n), dtype=torch.complex128, device="cuda")
        hc = torch.zeros((len(MODES), n), dtype=torch.complex128, device="cuda")
        tf = torch.zeros((len(MODES), n), dtype=torch.float64, device="cuda")
        # views into one (6, n) block per field, so that the producer fills every mode in one call
        return {m: {"plus": hp[k], "cross": hc[k], "tf": tf[k]} for k, m in enumerate(MODES)}

    def _run(self, theta, out):
        theta = np.ascontiguousarray(theta, dtype=np.float64).copy()
        theta[10] = 0.0  # t_c is applied by the response
        first = out[MODES[0]]
        n = self.frequencies.numel()
        _lib.check(_lib.load().pes_phenomhm(
            _lib.ptr(theta), _lib.ptr(self.frequencies), n, self.reference_frequency,
            min(self.cutoff_frequency, 1e300), _lib.ptr(first["plus"]), _lib.ptr(first["cross"]),
            _lib.ptr(first["tf"]), _lib.stream_handle()))
        return out

    def update_waveform(self, parameters):
        """tiwave-style: fill ``waveform_container`` in place."""
        self._run(theta_from_parameters(parameters), self.waveform_container)

    def get_waveform(self, params):
        """ripple-style: return a fresh mode-keyed container."""
        return self._run(theta_from_parameters(params), self._empty())

    def from_theta(self, theta):
        return self._run(theta, self._empty())

    __call__ = get_waveform
