"""The package's own host set-up path (the one bench.py and the likelihood
engines build their data with) against the reference's outputs in
tests/golden/: the dense grid, the analytic PSDs and the seeded noise
realisation, bit for bit.  CPU only (NumPy; no device needed)."""

import numpy as np
import pytest

from pespace_gb300.constants import C_SI
from pespace_gb300.detector.noise import TianQinAnalyticPowerSpectralDensity, available_noise_models
from pespace_gb300.detector.tdi import DataInformation, fd_noise_realization_array

# the golden PSD cases: three presets of noise.py:268-284 and TianQin at L = sqrt(3) 1e8 m
MODELS = {
    "lisa": available_noise_models["LISA_SciRDv1"],
    "taiji": available_noise_models["Taiji_TDC"],
    "tianqin_gwspace": available_noise_models["Tianqin_GWSpace"],
    "tianqin_sqrt3": TianQinAnalyticPowerSpectralDensity(1e-24, 1e-30, np.sqrt(3.0) * 1e8 / C_SI),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("scaling", [0, 1])
def test_psd_bit_exact(golden, name, gen, scaling):
    d = MODELS[name](golden["psd_freqs"], tuple("XYZAET"), bool(scaling), gen)
    np.testing.assert_array_equal(np.stack([d[c] for c in "XYZAET"]), golden[f"psd_{name}_{gen}_{scaling}"])


def test_grid_bit_exact(golden):
    for i, (dur, dt, fmin, fmax) in enumerate(golden["grid_cases"]):
        info = DataInformation(("A", "E", "T"), float(dur), float(dt), 0.0, float(fmin), float(fmax))
        meta = golden[f"grid{i}_meta"]
        assert (info.time_series_length, info.full_frequency_series_length, info.frequency_series_length) == tuple(
            int(x) for x in meta[:3])
        assert info.delta_frequency == meta[3]
        fk = info.frequency_samples_array
        if f"grid{i}_freqs" in golden.files:
            np.testing.assert_array_equal(fk, golden[f"grid{i}_freqs"])
        else:
            np.testing.assert_array_equal(fk[:32], golden[f"grid{i}_freqs_head"])
            np.testing.assert_array_equal(fk[-32:], golden[f"grid{i}_freqs_tail"])
            np.testing.assert_array_equal(fk[::997], golden[f"grid{i}_freqs_stride997"])
        if info.frequency_series_length:
            # the kernels' f_k = (k0 + i) f_step reproduces the masked rfftfreq grid
            idx = info.first_index + np.arange(info.frequency_series_length)
            np.testing.assert_array_equal(idx * info.frequency_step, fk)


def test_noise_psd_and_realisation_bit_exact(golden):
    info = DataInformation(("A", "E", "T"), 2.0 ** 15, 8.0, 0.0, 1e-4, 0.03)
    d = available_noise_models["LISA_SciRDv1"](info.frequency_samples_array, info.channels, False, "1.5")
    psd = np.stack([d[c] for c in "AET"])
    np.testing.assert_array_equal(psd, golden["noise_psd_lisa_15"])
    noise = fd_noise_realization_array(info, psd, 2026)
    np.testing.assert_array_equal(noise, golden["noise_seed2026_lisa_15"])
    # another seed draws another realisation
    assert not np.array_equal(fd_noise_realization_array(info, psd, 2027), noise)
