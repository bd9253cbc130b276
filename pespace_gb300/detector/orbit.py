"""Orbit models (pespace/detector/orbit.py) with the CUDA backend.

``KaplerianHeliocentric`` (LISA/Taiji) and ``KeplerianGeocentric`` (TianQin)
keep the reference constructors, ``orbit_params`` fields and methods
(orbit.py:77-152, 166-241); ``get_constellation_vectors`` runs the
``pes_orbit_vectors`` kernel.
"""

from collections import namedtuple

import numpy as np
import torch

from .. import _lib
from ..constants import C_SI, DAY_SI, PI, YEAR_SI

ConstellationVectorTuple = namedtuple("ConstellationVectorTuple", ["n1", "n2", "n3", "x1", "x2", "x3"])


class OrbitModelBase:
    """Base class of the analytic constellation orbits (orbit.py:27-64)."""

    backend = "cuda"

    def get_constellation_vectors(self, time):
        time_t = torch.as_tensor(time, dtype=torch.float64, device="cuda")
        flat = time_t.reshape(-1).contiguous()
        out = torch.empty((flat.numel(), 6, 3), dtype=torch.float64, device="cuda")
        desc = self.to_c()
        _lib.check(_lib.load().pes_orbit_vectors(desc, _lib.ptr(flat), flat.numel(), _lib.ptr(out),
                                                 _lib.stream_handle()))
        out = out.reshape(*time_t.shape, 6, 3)
        return ConstellationVectorTuple(*[out[..., i, :] for i in range(6)])

    def arm_length_sec(self, time=0.0):
        return self.orbit_params.static_arm_sec


class KeplerianGeocentric(OrbitModelBase):
    """Analytic Keplerian geocentric orbit (TianQin); orbit.py:67-152."""

    def __init__(self, arm_length, rotation_initial=0.0, revolution_initial=0.0,
                 omega_rotation=2 * PI / (3.65 * DAY_SI), lambda_ref=120.5 / 180 * PI,
                 beta_ref=-4.7 / 180 * PI, backend="cuda"):
        if backend != "cuda":
            raise ValueError(f"Unknown backend: {backend}")
        OrbitParams = namedtuple("OrbitParams", ["static_arm_sec", "r_det_sec", "rotation_initial",
                                                 "revolution_initial", "omega_rotation", "omega_revolution",
                                                 "slam_ref", "clam_ref", "sbeta_ref", "cbeta_ref"])
        self.orbit_params = OrbitParams(
            static_arm_sec=arm_length / C_SI,
            r_det_sec=arm_length / C_SI / np.sqrt(3),
            rotation_initial=rotation_initial,
            revolution_initial=revolution_initial,
            omega_rotation=omega_rotation,
            omega_revolution=2 * PI / YEAR_SI,
            slam_ref=np.sin(lambda_ref),
            clam_ref=np.cos(lambda_ref),
            sbeta_ref=np.sin(beta_ref),
            cbeta_ref=np.cos(beta_ref),
        )
        self.backend = backend

    def to_c(self):
        p = self.orbit_params
        o = _lib.PesOrbit()
        o.kind = 1
        o.arm_sec = p.static_arm_sec
        o.rotation_initial = p.rotation_initial
        o.revolution_initial = p.revolution_initial
        o.omega_revolution = p.omega_revolution
        o.r_sec = p.r_det_sec
        o.omega_rotation = p.omega_rotation
        o.slam_ref, o.clam_ref, o.sbeta_ref, o.cbeta_ref = p.slam_ref, p.clam_ref, p.sbeta_ref, p.cbeta_ref
        return o


class KaplerianHeliocentric(OrbitModelBase):
    """Analytic Keplerian heliocentric orbit (LISA, Taiji); orbit.py:155-241."""

    def __init__(self, arm_length, rotation_initial=0.0, revolution_initial=0.0, backend="cuda"):
        if backend != "cuda":
            raise ValueError(f"Unknown backend: {backend}")
        arm_sec = arm_length / C_SI
        k1 = rotation_initial
        k2 = k1 + 2 * PI / 3
        k3 = k2 + 2 * PI / 3
        OrbitParams = namedtuple("OrbitParams", ["static_arm_sec", "rotation_initial", "revolution_initial",
                                                 "r_prime", "omega", "ck1", "sk1", "ck2", "sk2", "ck3", "sk3"])
        self.orbit_params = OrbitParams(
            static_arm_sec=arm_sec,
            rotation_initial=rotation_initial,
            revolution_initial=revolution_initial,
            r_prime=arm_sec / (2 * np.sqrt(3)),
            omega=2 * PI / YEAR_SI,
            ck1=np.cos(k1), sk1=np.sin(k1), ck2=np.cos(k2), sk2=np.sin(k2), ck3=np.cos(k3), sk3=np.sin(k3),
        )
        self.backend = backend

    def to_c(self):
        p = self.orbit_params
        o = _lib.PesOrbit()
        o.kind = 0
        o.arm_sec = p.static_arm_sec
        o.rotation_initial = p.rotation_initial
        o.revolution_initial = p.revolution_initial
        o.omega_revolution = p.omega
        o.r_sec = p.r_prime
        for j, (c, s) in enumerate(((p.ck1, p.sk1), (p.ck2, p.sk2), (p.ck3, p.sk3))):
            o.ck[j] = c
            o.sk[j] = s
        return o


# orbit.py:442-446 presets
available_orbit_models = {
    "LISA_analytic": lambda: KaplerianHeliocentric(2.5e9, 0.0, -PI / 9),
    "Taiji_analytic": lambda: KaplerianHeliocentric(3.0e9, 0.0, PI / 9),
    "Tianqin_analytic": lambda: KeplerianGeocentric(1.7e8, 0.0, 0.0),
}
