"""Analytic noise PSDs of pespace/detector/noise.py (host-side set-up, NumPy).

The PSD is evaluated once per dataset on the host, exactly as the reference
does; it then lives on the device as inverse PSD inside the likelihood plan.
"""

from dataclasses import dataclass

import numpy as np
from numpy import cos, sin

from ..constants import C_SI, MRSUN_SI, MTSUN_SI, PC_SI, PI


class FrequencyDomainNoiseModel:
    """noise.py:12-45: callable PSD model."""

    def __call__(self, frequencies, tdi_channels, scaling, tdi_generation):
        return self.power_spectral_density_array(frequencies, tdi_channels, scaling, tdi_generation)


@dataclass
class AnalyticPowerSpectralDensity(FrequencyDomainNoiseModel):
    """noise.py:48-207 (arXiv:2108.01167 model)."""

    OMS_noise_level: float
    acc_noise_level: float
    arm_length_sec: float

    def _S_oms(self, f):
        return self.OMS_noise_level * (1.0 + (2.0e-3 / f) ** 4) * (2.0 * PI * f / C_SI) ** 2

    def _S_acc(self, f):
        return self.acc_noise_level * (1.0 + (0.4e-3 / f) ** 2) * (1.0 + (f / 8e-3) ** 4) / (2 * PI * f * C_SI) ** 2

    def power_spectral_density_array(self, frequencies, tdi_channels, scaling, tdi_generation):
        f = np.asarray(frequencies, dtype=np.float64)
        S_oms = self._S_oms(f)
        S_acc = self._S_acc(f)
        if scaling:
            sf = (PC_SI / (MRSUN_SI * MTSUN_SI)) ** 2
            S_oms = S_oms * sf
            S_acc = S_acc * sf
        if tdi_generation == "1.5":
            pre = 1.0
        elif tdi_generation == "2.0":
            pre = 4.0 * sin(4 * PI * f * self.arm_length_sec) ** 2
        else:
            raise ValueError("The TDI generation {} is unknown".format(tdi_generation))
        L = self.arm_length_sec
        out = {}
        for chan in tdi_channels:
            if chan in ("X", "Y", "Z"):
                psd = 16 * sin(2 * PI * f * L) ** 2 * (S_oms + (3 + cos(4 * PI * f * L)) * S_acc)
            elif chan in ("A", "E"):
                psd = 8 * sin(2 * PI * f * L) ** 2 * (
                    (2 + cos(2 * PI * f * L)) * S_oms
                    + (6 + 4 * cos(2 * PI * f * L) + 2 * cos(4 * PI * f * L)) * S_acc)
            elif chan == "T":
                psd = 32 * sin(2 * PI * f * L) ** 2 * sin(PI * f * L) ** 2 * (
                    S_oms + 4 * sin(PI * f * L) ** 2 * S_acc)
            else:
                raise ValueError(f"Unknown TDI channel {chan}.")
            out[chan] = psd * pre
        return out


class TianQinAnalyticPowerSpectralDensity(AnalyticPowerSpectralDensity):
    """noise.py:210-265 (arXiv:2309.15020 model)."""

    def _S_oms(self, f):
        return self.OMS_noise_level * (2.0 * PI * f / C_SI) ** 2

    def _S_acc(self, f):
        return self.acc_noise_level * (1.0 + 0.1e-3 / f) / (2 * PI * f * C_SI) ** 2


available_noise_models = {
    "LISA_SciRDv1": AnalyticPowerSpectralDensity((15.0e-12) ** 2, (3.0e-15) ** 2, 2.5e9 / C_SI),
    "Taiji_TDC": AnalyticPowerSpectralDensity((8.0e-12) ** 2, (3.0e-15) ** 2, 3.0e9 / C_SI),
    "Tianqin_GWSpace": TianQinAnalyticPowerSpectralDensity((1.0e-12) ** 2, (1.0e-15) ** 2, 1.7e8 / C_SI),
}
