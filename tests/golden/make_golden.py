"""Generate the golden fixtures of the FD response / TDI / Whittle-likelihood path.

Every output array in ``reference_fd_path.npz`` is computed by the reference
package itself (nnrui/pespace), imported from a checkout given on the command
line, through its JAX backend with NumPy standing in for ``jax.numpy``
(``_refshim.py``).  The reference notebooks show that backend agreeing with the
taichi backend to ~1e-12 relative (examples/_checks/likelihood_jax.ipynb cell 20,
examples/_checks/response_jax.ipynb cell 13).

Inputs (waveform containers, sky angles, grids) are synthetic and seeded; the
waveform is a leading-order chirp written here, not PhenomD, because the
response/TDI/likelihood stages take any ``{"plus", "cross", "tf"}`` container.

Usage (needs the reference checkout; the fixture is committed):

    python tests/golden/make_golden.py /path/to/pespace-checkout
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _refshim  # noqa: E402

MTSUN_SI = 4.925490947641266978197229498498379006e-6


def toy_chirp(freqs, mtot_msun, eta, amp0, phi0, zero_above):
    """Leading-order (Newtonian) SPA chirp: plus/cross polarisations and t(f)."""
    m_sec = mtot_msun * MTSUN_SI
    v = (np.pi * m_sec * freqs) ** (1.0 / 3.0)
    psi = 3.0 / (128.0 * eta) * v ** (-5) - phi0
    tf = -5.0 / (256.0 * eta) * m_sec * v ** (-8)
    amp = amp0 * freqs ** (-7.0 / 6.0)
    amp = np.where(freqs <= zero_above, amp, 0.0)
    tf = np.where(freqs <= zero_above, tf, 0.0)
    h = amp * np.exp(-1j * psi)
    cosi = np.cos(0.6)
    return {
        "plus": h * 0.5 * (1.0 + cosi**2),
        "cross": -1j * cosi * h,
        "tf": tf,
    }


def main(ref_root):
    _refshim.install(ref_root)
    from collections import namedtuple

    from pespace.detector import orbit as r_orbit
    from pespace.detector import antenna as r_antenna
    from pespace.detector import tdi as r_tdi
    from pespace.detector import noise as r_noise
    from pespace.detector._jax_impl import _antenna_jax
    from pespace.inference import likelihood_jax as r_lik
    from pespace.waveform.interface_ripple import WaveformRippleBase
    from pespace.utils.constants import PI, C_SI

    out = {}
    rng = np.random.default_rng(20260)

    # ---------------------------------------------------------------- orbits
    times = np.concatenate([[0.0, -3.0e6, 1.0e5], rng.uniform(-4e7, 4e7, 13)])
    out["orbit_times"] = times
    orbits = {
        "lisa": r_orbit.KaplerianHeliocentric(2.5e9, 0.0, -PI / 9, backend="jax"),
        "taiji": r_orbit.KaplerianHeliocentric(3.0e9, 0.0, PI / 9, backend="jax"),
        "tianqin": r_orbit.KeplerianGeocentric(np.sqrt(3.0) * 1e8, 0.3, 0.2, backend="jax"),
        "helio_rot": r_orbit.KaplerianHeliocentric(2.5e9, 0.7, 1.1, backend="jax"),
    }
    for name, orb in orbits.items():
        vec = orb.get_constellation_vectors(times)
        out[f"orbit_{name}"] = np.stack(
            [vec.n1, vec.n2, vec.n3, vec.x1, vec.x2, vec.x3], axis=1
        )  # (T, 6, 3)
        out[f"orbit_{name}_arm"] = np.array(orb.arm_length_sec(0.0))

    # ------------------------------------------------------ polarisation, k
    angles = np.stack(
        [rng.uniform(0, 2 * np.pi, 8), rng.uniform(-1.5, 1.5, 8), rng.uniform(0, np.pi, 8)],
        axis=1,
    )
    out["pol_angles"] = angles
    plus, cross, kvec = [], [], []
    for lam, beta, psi in angles:
        pol = _antenna_jax.get_polarization_tensor_ssb_jax(lam, beta, psi)
        plus.append(pol.plus)
        cross.append(pol.cross)
        kvec.append(_antenna_jax.get_gw_propagation_unit_vector_jax(lam, beta))
    out["pol_plus"] = np.array(plus)
    out["pol_cross"] = np.array(cross)
    out["prop_k"] = np.array(kvec)

    # ------------------------------------------------------------ grids
    grid_cases = [
        (2.0**15, 8.0, 1e-4, 0.03),
        (2.0**22, 8.0, 1e-4, 0.03),
        (655360.0, 5.0, 1e-4, 0.1),
        (1000.0, 3.0, 1e-3, 0.15),
        (2.0**12, 16.0, 0.0, 1.0),
    ]
    out["grid_cases"] = np.array(grid_cases)
    for i, (dur, dt, fmin, fmax) in enumerate(grid_cases):
        info = r_tdi.DataInformation(("A", "E", "T"), dur, dt, 0.0, fmin, fmax)
        fs = info.frequency_samples_array
        if fs.size <= 5000:
            out[f"grid{i}_freqs"] = fs
        else:  # large grids: keep the ends and every 997th sample
            out[f"grid{i}_freqs_head"] = fs[:32]
            out[f"grid{i}_freqs_tail"] = fs[-32:]
            out[f"grid{i}_freqs_stride997"] = fs[::997]
        out[f"grid{i}_meta"] = np.array(
            [
                info.time_series_length,
                info.full_frequency_series_length,
                info.frequency_series_length,
                info.delta_frequency,
                int(np.argmax(info.frequency_mask_array)) if info.frequency_series_length else -1,
            ],
            dtype=np.float64,
        )

    # ------------------------------------------------------------- PSDs
    psd_f = np.geomspace(3e-5, 0.5, 301)
    out["psd_freqs"] = psd_f
    psd_models = {
        "lisa": r_noise.available_noise_models["LISA_SciRDv1"],
        "taiji": r_noise.available_noise_models["Taiji_TDC"],
        "tianqin_gwspace": r_noise.available_noise_models["Tianqin_GWSpace"],
        "tianqin_sqrt3": r_noise.TianQinAnalyticPowerSpectralDensity(
            OMS_noise_level=(1.0e-12) ** 2,
            acc_noise_level=(1.0e-15) ** 2,
            arm_length_sec=np.sqrt(3.0) * 1e8 / C_SI,
        ),
    }
    for name, model in psd_models.items():
        for gen in ("1.5", "2.0"):
            for scaling in (False, True):
                d = model(psd_f, ("X", "Y", "Z", "A", "E", "T"), scaling, gen)
                out[f"psd_{name}_{gen}_{int(scaling)}"] = np.stack(
                    [d[c] for c in ("X", "Y", "Z", "A", "E", "T")]
                )

    # ------------------------------------------- detectors on a small grid
    dur, dt, fmin, fmax = 2.0**15, 8.0, 1e-4, 0.03
    tc = 0.8 * dur
    det_specs = {
        "lisa": (orbits["lisa"], "LISA_SciRDv1", {}),
        "tianqin": (orbits["tianqin"], psd_models["tianqin_sqrt3"], {}),
    }

    def make_detector(orb, psd_model, gen, orth, with_noise_seed=None):
        data = r_tdi.TDIChannelData(scaling=False, backend="jax")
        labels = ("A", "E", "T") if orth else ("X", "Y", "Z")
        data.set_fd_data_from_zero(labels, dur, dt, 0.0, fmin, fmax)
        data.set_fd_noise_power_density_from_model(psd_model, tdi_generation=gen)
        det = r_antenna.InterferometerAntenna(
            "det",
            data,
            orb,
            r_antenna.FDResponseModelMarset2018(backend="jax"),
            r_tdi.FDMichelsonConstantEqualArm(gen, orth, backend="jax"),
            backend="jax",
        )
        return det

    freqs = None
    for dname, (orb, psd_model, _) in det_specs.items():
        for gen in ("1.5", "2.0"):
            for orth in (True, False):
                det = make_detector(orb, psd_model, gen, orth)
                freqs = np.asarray(det.tdi_data.frequency_samples)
                wf = toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, zero_above=0.02)
                lam, beta, psi = 1.0, 0.3, 0.7
                det.update_detector_response(wf, lam, beta, psi, tc)
                key = f"resp_{dname}_{gen}_{int(orth)}"
                out[key + "_links"] = np.stack(list(det.single_link_response))
                out[key + "_tdi"] = np.stack(list(det.tdi_response))
    out["resp_freqs"] = freqs
    out["resp_wf_plus"] = toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, 0.02)["plus"]
    out["resp_wf_cross"] = toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, 0.02)["cross"]
    out["resp_wf_tf"] = toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, 0.02)["tf"]
    out["resp_extrinsic"] = np.array([1.0, 0.3, 0.7, tc])

    # multi-mode container: mode-keyed dict, links summed over modes
    det = make_detector(orbits["lisa"], "LISA_SciRDv1", "2.0", True)
    wf22 = toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, 0.02)
    wf33 = toy_chirp(1.5 * freqs, 1.5e6, 0.2, 3e-22, 1.3, 0.02)
    wf33["tf"] = wf33["tf"] + 30.0
    modes = {"22": wf22, "33": wf33}
    det.update_detector_response(modes, 2.1, -0.4, 1.2, tc - 500.0)
    out["mm_wf_plus"] = np.stack([wf22["plus"], wf33["plus"]])
    out["mm_wf_cross"] = np.stack([wf22["cross"], wf33["cross"]])
    out["mm_wf_tf"] = np.stack([wf22["tf"], wf33["tf"]])
    out["mm_extrinsic"] = np.array([2.1, -0.4, 1.2, tc - 500.0])
    out["mm_links"] = np.stack(list(det.single_link_response))
    out["mm_tdi"] = np.stack(list(det.tdi_response))

    # --------------------------------------- noise realisation (seeded)
    det = make_detector(orbits["lisa"], "LISA_SciRDv1", "1.5", True)
    noise = det.tdi_data.get_fd_noise_realization(seed=2026, output_type="numpy")
    out["noise_seed2026_lisa_15"] = np.stack([noise.A, noise.E, noise.T])
    out["noise_psd_lisa_15"] = np.stack(list(det.tdi_data.fd_noise_power_density))

    # ---------------------------------------------- likelihood (full path)
    class FixedWaveform(WaveformRippleBase):
        """Waveform container source returning precomputed arrays by parameter set."""

        def __init__(self, frequencies, table):
            super().__init__(frequencies, 1e-4)
            self.table = table

        @property
        def required_params(self):
            return ("wf_index",)

        def get_waveform(self, params):
            return self.table[int(params.wf_index)]

    table = [
        toy_chirp(freqs, 1.5e6, 0.2, 1e-21, 0.4, 0.02),
        toy_chirp(freqs, 1.52e6, 0.2, 1.1e-21, 0.9, 0.02),
        toy_chirp(freqs, 1.2e6, 0.24, 0.7e-21, 2.2, 0.025),
    ]
    extr = [(1.0, 0.3, 0.7, tc), (1.05, 0.28, 0.8, tc + 12.0), (4.0, -0.9, 2.0, tc - 900.0)]
    lik_cases = []
    for gen in ("1.5", "2.0"):
        det_l = make_detector(orbits["lisa"], "LISA_SciRDv1", gen, True)
        det_t = make_detector(orbits["tianqin"], psd_models["tianqin_sqrt3"], gen, True)
        for d_i, det_i in enumerate((det_l, det_t)):
            n = det_i.tdi_data.get_fd_noise_realization(seed=2026 + d_i, output_type="numpy")
            det_i.tdi_data.add_into_fd_data(n)
            det_i.inject_signal(table[0], *extr[0])
        out[f"lik_{gen}_data_lisa"] = np.stack(list(det_l.tdi_data.fd_data))
        out[f"lik_{gen}_psd_lisa"] = np.stack(list(det_l.tdi_data.fd_noise_power_density))
        out[f"lik_{gen}_data_tianqin"] = np.stack(list(det_t.tdi_data.fd_data))
        out[f"lik_{gen}_psd_tianqin"] = np.stack(list(det_t.tdi_data.fd_noise_power_density))
        wfgen = FixedWaveform(det_l.tdi_data.frequency_samples, table)
        for chans in (("A", "E", "T"), ("A", "E"), ("T",)):
            for dets, dtag in (((det_l,), "lisa"), ((det_l, det_t), "net")):
                lik = r_lik.WhittleLikelihoodJax(wfgen, dets, chans)
                P = lik.likelihood_param_type
                for w_i, (lam, beta, psi, t_c) in enumerate(extr):
                    val = lik.log_likelihood(
                        P(
                            wf_index=w_i,
                            ecliptic_longitude=lam,
                            ecliptic_latitude=beta,
                            polarization=psi,
                            coalescence_time=t_c,
                        )
                    )
                    lik_cases.append((float(gen), len(chans), "AET".index(chans[0]), dtag == "net", w_i, float(val)))
    out["lik_cases"] = np.array(lik_cases)
    out["lik_extrinsic"] = np.array(extr)
    out["lik_wf_plus"] = np.stack([t["plus"] for t in table])
    out["lik_wf_cross"] = np.stack([t["cross"] for t in table])
    out["lik_wf_tf"] = np.stack([t["tf"] for t in table])

    # elementary Whittle kernel on random inputs
    dd = rng.normal(size=(3, 257)) + 1j * rng.normal(size=(3, 257))
    hh = rng.normal(size=(3, 257)) + 1j * rng.normal(size=(3, 257))
    ss = rng.uniform(0.5, 2.0, size=(3, 257))
    out["nwip_d"], out["nwip_h"], out["nwip_s"] = dd, hh, ss
    out["nwip_value"] = np.array(r_lik.noise_weighted_inner_product(dd, hh, ss, 0.125))

    path = os.path.join(HERE, "reference_fd_path.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes uncompressed")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path to the pespace checkout>")
    main(sys.argv[1])
