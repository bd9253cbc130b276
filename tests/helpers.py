"""Shared set-up for the parity tests: identical datasets for oracle and CUDA."""

import numpy as np

PI = np.pi


def config0_theta(tc):
    """Config-0 source: m1=1e6, m2=5e5 Msun, chi=(0.5,-0.3), 10 Gpc, iota=pi/3,
    lambda=1.0, beta=0.3, psi=0.7, phi_c=0."""
    m1, m2 = 1e6, 5e5
    q = m1 / m2
    eta = m1 * m2 / (m1 + m2) ** 2
    mc = (m1 + m2) * eta ** 0.6
    return np.array([np.log(mc), q, 0.5, -0.3, np.log(1e4), np.cos(PI / 3), 1.0, np.sin(0.3), 0.7, 0.0, tc])


def perturbed(theta, rng, scale=1.0):
    t = theta.copy()
    t[0] += 1e-4 * scale * rng.normal()
    t[1] = max(1.0, t[1] + 0.02 * scale * rng.normal())
    t[2] = np.clip(t[2] + 0.05 * scale * rng.normal(), -0.95, 0.95)
    t[3] = np.clip(t[3] + 0.05 * scale * rng.normal(), -0.95, 0.95)
    t[4] += 0.05 * scale * rng.normal()
    t[5] = np.clip(t[5] + 0.05 * scale * rng.normal(), -1, 1)
    t[6] += 0.05 * scale * rng.normal()
    t[7] = np.clip(t[7] + 0.05 * scale * rng.normal(), -1, 1)
    t[8] += 0.05 * scale * rng.normal()
    t[9] += 0.05 * scale * rng.normal()
    t[10] += 20.0 * scale * rng.normal()
    return t


def random_prior_theta(rng, B, tc0):
    """Batched-config prior: Mtot log-uniform 1e5..1e7, q U[1,8], chi U[-0.99,0.99],
    isotropic sky and inclination, psi/phi uniform, tc within 1 h, D_L 1..30 Gpc (uniform in volume)."""
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


def make_dataset(oracle, duration, dt, fmin, fmax, dets, theta_inj, seed=2026, f_ref=1e-4):
    """Injection (oracle FP64 model) + seeded noise per detector.

    dets: list of (name, orbit_desc, generation, psd_kwargs).  Returns the grid and
    per-detector (data (3,N) complex, psd (3,N)).
    """
    g = oracle.grid(duration, dt, fmin, fmax)
    out = []
    for i, (name, orb, gen, psd_kw) in enumerate(dets):
        psd = oracle.psd(g["freqs"], "AET", False, gen, **psd_kw)
        psd_arr = np.stack([psd[c] for c in "AET"])
        noise = oracle.noise_realization(g, psd, "AET", seed + i)
        data = np.stack([noise[c] for c in "AET"])
        out.append([name, orb, gen, data, psd_arr])
    # injection via the oracle model
    plan = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in out], f_ref)
    for i in range(len(out)):
        h = plan.model_tdi(i, theta_inj)
        out[i][3] = out[i][3] + h
    return g, out
