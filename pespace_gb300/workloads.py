"""Synthetic workloads of the benchmark configurations (seeded, no external data).

* ``config0_theta``: one IMRPhenomD MBHB, m1 = 1e6, m2 = 5e5 Msun (detector
  frame), chi = (0.5, -0.3), D_L = 10 Gpc, iota = pi/3, lambda = 1.0,
  beta = 0.3, psi = 0.7, phi_c = 0, t_c = T - 86400 s.
* ``prior_samples``: the batched-configuration prior (total mass log-uniform
  in 1e5..1e7 Msun, q in U[1, 8], spins U[-0.99, 0.99], isotropic sky and
  inclination, psi and phi_c uniform, t_c within +-1 h of the injection,
  D_L uniform in volume over 1..30 Gpc; Euclidean volume, no cosmology).
* ``lisa_dataset``: LISA-like heliocentric detector (L = 2.5e9 m, trailing
  20 deg), SciRDv1 PSD, A/E/T of a chosen TDI generation, data = injection +
  seeded noise (the reference recipe, pespace/detector/tdi.py:896-916).
"""

import math

import numpy as np

PI = math.pi


def config0_theta(tc):
    m1, m2 = 1e6, 5e5
    q = m1 / m2
    eta = m1 * m2 / (m1 + m2) ** 2
    mc = (m1 + m2) * eta ** 0.6
    return np.array([math.log(mc), q, 0.5, -0.3, math.log(1e4), math.cos(PI / 3), 1.0, math.sin(0.3), 0.7, 0.0, tc])


def prior_samples(rng, B, tc0):
    mtot = np.exp(rng.uniform(np.log(1e5), np.log(1e7), B))
    q = rng.uniform(1.0, 8.0, B)
    eta = q / (1 + q) ** 2
    mc = mtot * eta ** 0.6
    chi1 = rng.uniform(-0.99, 0.99, B)
    chi2 = rng.uniform(-0.99, 0.99, B)
    dl = (rng.uniform(1e3 ** 3, 3e4 ** 3, B)) ** (1 / 3)
    cosi = rng.uniform(-1, 1, B)
    lam = rng.uniform(0, 2 * PI, B)
    sinb = rng.uniform(-1, 1, B)
    psi = rng.uniform(0, PI, B)
    phi = rng.uniform(0, 2 * PI, B)
    tc = tc0 + rng.uniform(-3600, 3600, B)
    return np.stack([np.log(mc), q, chi1, chi2, np.log(dl), cosi, lam, sinb, psi, phi, tc], axis=1)


def lisa_dataset(duration, delta_time, fmin, fmax, theta_inj, generation="1.5", seed=2026, f_ref=1e-4,
                 arm_length=2.5e9, revolution_initial=-PI / 9, noise_model="LISA_SciRDv1", name="LISA"):
    """Build a CUDA ``InterferometerAntenna`` holding injection + noise."""
    from .detector.antenna import FDResponseModelMarset2018, InterferometerAntenna
    from .detector.orbit import KaplerianHeliocentric
    from .detector.tdi import FDMichelsonConstantEqualArm, TDIChannelData
    from .waveform import IMRPhenomD

    td = TDIChannelData()
    td.set_fd_data_from_zero(("A", "E", "T"), duration, delta_time, 0.0, fmin, fmax)
    td.set_fd_noise_power_density_from_model(noise_model, tdi_generation=generation)
    det = InterferometerAntenna(name, td, KaplerianHeliocentric(arm_length, 0.0, revolution_initial),
                                FDResponseModelMarset2018(), FDMichelsonConstantEqualArm(generation, True))
    td.add_into_fd_data(td.get_fd_noise_realization(seed=seed))
    wf = IMRPhenomD(td.data_info.frequency_samples_array, f_ref)
    th = np.asarray(theta_inj, dtype=np.float64)
    det.inject_signal(wf.from_theta(th), th[6], math.asin(th[7]), th[8], th[10])
    return det


def network_dataset(duration, delta_time, fmin, fmax, theta_inj, generation="1.5", seed=2026, f_ref=1e-4,
                    approximant="IMRPhenomD"):
    """Three-detector network of the higher-mode benchmark configuration:
    LISA-like (2.5e9 m, trailing 20 deg), Taiji-like (3e9 m, leading 20 deg;
    OMS 8e-12, acceleration 3e-15) and TianQin-like geocentric (sqrt(3) 1e8 m;
    OMS 1e-12, acceleration 1e-15); seeded noise per detector (seed, seed + 1,
    seed + 2) plus the injection of ``approximant`` (IMRPhenomD's (2,2) mode,
    or the six IMRPhenomHM modes)."""
    from .detector.antenna import FDResponseModelMarset2018, InterferometerAntenna
    from .detector.orbit import KaplerianHeliocentric, KeplerianGeocentric
    from .detector.tdi import FDMichelsonConstantEqualArm, TDIChannelData
    from .waveform import IMRPhenomD, IMRPhenomHM

    specs = [("LISA", KaplerianHeliocentric(2.5e9, 0.0, -PI / 9), "LISA_SciRDv1"),
             ("Taiji", KaplerianHeliocentric(3.0e9, 0.0, PI / 9), "Taiji_TDC"),
             ("TianQin", KeplerianGeocentric(math.sqrt(3.0) * 1e8), "Tianqin_GWSpace")]
    th = np.asarray(theta_inj, dtype=np.float64)
    dets = []
    for k, (name, orbit, noise) in enumerate(specs):
        td = TDIChannelData()
        td.set_fd_data_from_zero(("A", "E", "T"), duration, delta_time, 0.0, fmin, fmax)
        td.set_fd_noise_power_density_from_model(noise, tdi_generation=generation)
        det = InterferometerAntenna(name, td, orbit, FDResponseModelMarset2018(),
                                    FDMichelsonConstantEqualArm(generation, True))
        td.add_into_fd_data(td.get_fd_noise_realization(seed=seed + k))
        wf = (IMRPhenomHM if approximant == "IMRPhenomHM" else IMRPhenomD)(td.data_info.frequency_samples_array, f_ref)
        det.inject_signal(wf.from_theta(th), th[6], math.asin(th[7]), th[8], th[10])
        dets.append(det)
    return tuple(dets)
