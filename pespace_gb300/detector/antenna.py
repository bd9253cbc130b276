"""Detector aggregate and FD single-link response (pespace/detector/antenna.py).

``FDResponseModelMarset2018.update_single_link_response(waveform, lam, beta,
psi, tc)`` runs the ``pes_response_links`` kernel over the detector's
frequency grid.  The waveform container is a dict ``{"plus", "cross", "tf"}``
of CUDA tensors, or a mode-keyed dict of such dicts (antenna.py:438-458).
"""

from abc import ABC, abstractmethod

import torch

from .. import _lib
from .orbit import OrbitModelBase, available_orbit_models


def get_polarization_tensor_ssb(lam, beta, psi):
    """antenna.py:42-87: (e+, ex) as 3x3 NumPy arrays."""
    import numpy as np

    plus = np.zeros((3, 3))
    cross = np.zeros((3, 3))
    k = np.zeros(3)
    _lib.check(_lib.load().pes_polarization(float(lam), float(beta), float(psi), _lib.ptr(plus), _lib.ptr(cross),
                                            _lib.ptr(k)))
    return plus, cross


def get_gw_propagation_unit_vector(lam, beta):
    """antenna.py:90-114."""
    import numpy as np

    plus = np.zeros((3, 3))
    cross = np.zeros((3, 3))
    k = np.zeros(3)
    _lib.check(_lib.load().pes_polarization(float(lam), float(beta), 0.0, _lib.ptr(plus), _lib.ptr(cross),
                                            _lib.ptr(k)))
    return k


def _modes(waveform):
    if "plus" in waveform:
        return [waveform]
    return list(waveform.values())


class SingleLinkResponseModel(ABC):
    """antenna.py:326-344: the response plugin interface."""

    @abstractmethod
    def init_single_link_response_model(self, detector):
        pass

    @abstractmethod
    def update_single_link_response(self, waveform, lam, beta, psi, tc):
        pass


class FDResponseModelMarset2018(SingleLinkResponseModel):
    """antenna.py:347-543: Marsat et al. (2018) FD response, CUDA backend."""

    def __init__(self, backend="cuda"):
        if backend != "cuda":
            raise ValueError(f"Invalid backend: {backend}")
        self.backend = backend
        self.detector = None

    def init_single_link_response_model(self, detector):
        self.detector = detector
        n = detector.tdi_data.data_info.frequency_series_length
        detector.single_link_response = torch.zeros((6, n), dtype=torch.complex128, device="cuda")

    def update_single_link_response(self, waveform, lam, beta, psi, tc):
        det = self.detector
        freqs = det.tdi_data.frequency_samples
        n = freqs.numel()
        modes = _modes(waveform)
        hp = torch.stack([torch.as_tensor(m["plus"], dtype=torch.complex128, device="cuda") for m in modes])
        hc = torch.stack([torch.as_tensor(m["cross"], dtype=torch.complex128, device="cuda") for m in modes])
        tf = torch.stack([torch.as_tensor(m["tf"], dtype=torch.float64, device="cuda") for m in modes])
        if hp.shape[-1] != n:
            raise ValueError(f"waveform length {hp.shape[-1]} differs from the frequency grid ({n})")
        hp, hc, tf = hp.contiguous(), hc.contiguous(), tf.contiguous()
        _lib.check(_lib.load().pes_response_links(
            det.orbit_model.to_c(), _lib.ptr(freqs), n, len(modes), _lib.ptr(hp), _lib.ptr(hc), _lib.ptr(tf),
            float(lam), float(beta), float(psi), float(tc), _lib.ptr(det.single_link_response),
            _lib.stream_handle()))


class FDResponseModelLongWavelength(SingleLinkResponseModel):
    """antenna.py:546-553: a placeholder in the reference, as here (abstract:
    instantiating it raises TypeError, as there)."""


class FDResponseModelStaticLongWavelength(SingleLinkResponseModel):
    """antenna.py:556-563: a placeholder in the reference, as here (abstract:
    instantiating it raises TypeError, as there)."""


class InterferometerAntenna:
    """antenna.py:117-323: binds data, orbit, response and TDI models."""

    def __init__(self, name, tdi_data, orbit_model, response_model, tdi_combination, backend="cuda"):
        if backend != "cuda":
            raise ValueError(f"Unknown backend: {backend}")
        if isinstance(orbit_model, str):
            try:
                orbit_model = available_orbit_models[orbit_model]()
            except KeyError:
                raise ValueError(f"{orbit_model} is not a implemented orbit model. \n"
                                 f"Current available models are {[*available_orbit_models.keys()]}")
        if not isinstance(orbit_model, OrbitModelBase):
            raise TypeError(f"Expected OrbitModelBase or str for orbit_model, but got {type(orbit_model).__name__}.")
        for component in (tdi_data, orbit_model, response_model, tdi_combination):
            if getattr(component, "backend") != backend:
                raise ValueError(f"Backend mismatch: the passed class {component.__class__.__name__} uses "
                                 f"{component.backend} as its backend, but InterferometerAntenna uses {backend}.")
        self.name = name
        self.tdi_data = tdi_data
        self.orbit_model = orbit_model
        self.response_model = response_model
        self.tdi_combination = tdi_combination
        self.backend = backend
        self.tdi_response = None
        self.single_link_response = None
        self.tdi_combination.init_tdi_combination_model(self)
        self.response_model.init_single_link_response_model(self)

    def update_detector_response(self, waveform, lam, beta, psi, tc):
        self.response_model.update_single_link_response(waveform, lam, beta, psi, tc)
        self.tdi_combination.update_tdi_response()

    def inject_signal(self, waveform, lam, beta, psi, tc):
        self.update_detector_response(waveform, lam, beta, psi, tc)
        if self.tdi_combination.domain != "fd":
            raise NotImplementedError(f"Unsupported domain {self.tdi_combination.domain}")
        self.tdi_data.add_into_fd_data(self.tdi_response)

    def get_optimal_snr(self, waveform, lam, beta, psi, tc):
        """Optimal SNR per TDI channel and in total (antenna.py:273-303, a
        placeholder in the reference, which documents this return value).

        rho_c^2 = 4 df sum_f |h_c(f)|^2 / S_c(f) over the data's channels: the
        normalisation of the reference's likelihood, lnL = -2 df sum |d - h|^2
        / S.  Bins where S = 0 (the TDI zeros) contribute nothing.  The
        detector's response buffers hold this waveform's response afterwards.
        Returns {channel: rho_c, ..., "total": sqrt(sum_c rho_c^2)}.
        """
        if self.tdi_combination.domain != "fd":
            raise NotImplementedError(f"Unsupported domain {self.tdi_combination.domain}")
        psd = self.tdi_data.fd_noise_power_density
        if psd is None:
            raise ValueError("Setting `fd_noise_power_density` before computing the optimal SNR.")
        self.update_detector_response(waveform, lam, beta, psi, tc)
        df = float(self.tdi_data.data_info.delta_frequency)
        out, total = {}, 0.0
        for c_i, chan in enumerate(self.tdi_data.data_info.channels):
            h = self.tdi_response[self.tdi_combination.labels.index(chan)]
            S = psd[c_i]
            w = torch.where(S > 0, 1.0 / torch.where(S > 0, S, torch.ones_like(S)), torch.zeros_like(S))
            rho2 = 4.0 * df * float(torch.sum((h.real ** 2 + h.imag ** 2) * w).item())
            out[chan] = rho2 ** 0.5
            total += rho2
        out["total"] = total ** 0.5
        return out

    @property
    def tdi_response_numpy(self):
        from collections import namedtuple

        return namedtuple("DataContent", self.tdi_combination.labels)(*self.tdi_response.cpu().numpy())

    @property
    def single_link_response_array(self):
        from collections import namedtuple

        names = ("link12", "link21", "link23", "link32", "link31", "link13")
        return namedtuple("DataContent", names)(*self.single_link_response.cpu().numpy())
