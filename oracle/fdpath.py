"""Python side of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The CUDA product in ``pespace_gb300`` never imports this module.  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it,
as the checker.

It holds
* NumPy restatements of the reference's host-side set-up code: the dense
  frequency grid (pespace/detector/tdi.py:120-159), the analytic PSDs
  (pespace/detector/noise.py:71-207, 231-265, presets 268-284) and the seeded
  noise realisation (pespace/detector/tdi.py:896-916);
* ctypes bindings of ``pes_oracle.cpp`` (orbits, polarisation, single-link
  response, TDI, Whittle likelihood, IMRPhenomD, batched lnL and gradient).
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

PI = 3.141592653589793238462643383279502884
C_SI = 299792458.0
MRSUN_SI = 1.476625038050124729627979840144936351e3
MTSUN_SI = 4.925490947641266978197229498498379006e-6
YEAR_SI = 31557600.0
DAY_SI = 86400.0
AU_SI = 149597870700.0
PC_SI = 3.085677581491367e16


# ------------------------------------------------------------------ build/load
def build():
    """Compile ``pes_oracle.cpp`` into ``oracle/_build/liboracle.so``."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


class OrbitDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("arm_sec", ctypes.c_double),
        ("rotation_initial", ctypes.c_double),
        ("revolution_initial", ctypes.c_double),
        ("omega_revolution", ctypes.c_double),
        ("r_sec", ctypes.c_double),
        ("omega_rotation", ctypes.c_double),
        ("slam_ref", ctypes.c_double),
        ("clam_ref", ctypes.c_double),
        ("sbeta_ref", ctypes.c_double),
        ("cbeta_ref", ctypes.c_double),
        ("ck", ctypes.c_double * 3),
        ("sk", ctypes.c_double * 3),
    ]


class OracleDet(ctypes.Structure):
    _fields_ = [
        ("orbit", OrbitDesc),
        ("gen20", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("data", ctypes.c_void_p),
        ("psd", ctypes.c_void_p),
    ]


class OraclePlan(ctypes.Structure):
    _fields_ = [
        ("nbins", ctypes.c_int64),
        ("k0", ctypes.c_int64),
        ("f_step", ctypes.c_double),
        ("df", ctypes.c_double),
        ("f_ref", ctypes.c_double),
        ("cut_factor", ctypes.c_double),
        ("n_det", ctypes.c_int32),
        ("chan_mask", ctypes.c_int32),
        ("dets", ctypes.c_void_p),
        ("approximant", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


APPROXIMANTS = {"IMRPhenomD": 0, "IMRPhenomHM": 1}
HM_MODES = ((2, 2), (2, 1), (3, 3), (3, 2), (4, 4), (4, 3))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        d = ctypes.c_double
        i64 = ctypes.c_int64
        vp = ctypes.c_void_p
        L.oracle_orbit.argtypes = [P(OrbitDesc), vp, i64, vp]
        L.oracle_polarization.argtypes = [d, d, d, vp, vp, vp]
        L.oracle_response_links.argtypes = [P(OrbitDesc), vp, i64, ctypes.c_int, vp, vp, vp, d, d, d, d, vp]
        L.oracle_tdi.argtypes = [vp, i64, d, ctypes.c_int, ctypes.c_int, vp, vp]
        L.oracle_whittle.argtypes = [vp, vp, vp, ctypes.c_int, i64, d]
        L.oracle_whittle.restype = d
        L.oracle_phenomd.argtypes = [vp, vp, i64, d, d, vp, vp, vp, vp, vp]
        L.oracle_phenomhm.argtypes = [vp, vp, i64, d, d, vp, vp, vp, vp, vp]
        L.oracle_model_tdi.argtypes = [P(OraclePlan), ctypes.c_int, ctypes.c_int, vp, vp]
        L.oracle_lnl_batch.argtypes = [P(OraclePlan), vp, i64, vp, vp, ctypes.c_int]
        L.oracle_fisher_batch.argtypes = [P(OraclePlan), vp, i64, vp, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ------------------------------------------------------------------ orbits
def heliocentric(arm_length, rotation_initial=0.0, revolution_initial=0.0):
    """pespace/detector/orbit.py:166-229 (KaplerianHeliocentric)."""
    o = OrbitDesc()
    o.kind = 0
    o.arm_sec = arm_length / C_SI
    o.rotation_initial = rotation_initial
    o.revolution_initial = revolution_initial
    o.omega_revolution = 2 * PI / YEAR_SI
    o.r_sec = o.arm_sec / (2 * np.sqrt(3))
    k1 = rotation_initial
    k2 = k1 + 2 * PI / 3
    k3 = k2 + 2 * PI / 3
    for j, kap in enumerate((k1, k2, k3)):
        o.ck[j] = np.cos(kap)
        o.sk[j] = np.sin(kap)
    return o


def geocentric(arm_length, rotation_initial=0.0, revolution_initial=0.0,
               omega_rotation=2 * PI / (3.65 * DAY_SI), lambda_ref=120.5 / 180 * PI,
               beta_ref=-4.7 / 180 * PI):
    """pespace/detector/orbit.py:77-140 (KeplerianGeocentric)."""
    o = OrbitDesc()
    o.kind = 1
    o.arm_sec = arm_length / C_SI
    o.rotation_initial = rotation_initial
    o.revolution_initial = revolution_initial
    o.omega_revolution = 2 * PI / YEAR_SI
    o.r_sec = arm_length / C_SI / np.sqrt(3)
    o.omega_rotation = omega_rotation
    o.slam_ref = np.sin(lambda_ref)
    o.clam_ref = np.cos(lambda_ref)
    o.sbeta_ref = np.sin(beta_ref)
    o.cbeta_ref = np.cos(beta_ref)
    return o


def orbit_vectors(desc, times):
    times = np.ascontiguousarray(times, dtype=np.float64)
    out = np.zeros((times.size, 6, 3))
    lib().oracle_orbit(ctypes.byref(desc), _p(times), times.size, _p(out))
    return out


def polarization(lam, beta, psi):
    plus = np.zeros((3, 3))
    cross = np.zeros((3, 3))
    k = np.zeros(3)
    lib().oracle_polarization(lam, beta, psi, _p(plus), _p(cross), _p(k))
    return plus, cross, k


def response_links(desc, freqs, hp, hc, tf, lam, beta, psi, tc):
    """Single-link responses (6, n) for a (modes, n) waveform container."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    hp = np.ascontiguousarray(np.atleast_2d(hp), dtype=np.complex128)
    hc = np.ascontiguousarray(np.atleast_2d(hc), dtype=np.complex128)
    tf = np.ascontiguousarray(np.atleast_2d(tf), dtype=np.float64)
    out = np.zeros((6, freqs.size), dtype=np.complex128)
    lib().oracle_response_links(ctypes.byref(desc), _p(freqs), freqs.size, hp.shape[0], _p(hp), _p(hc), _p(tf),
                                lam, beta, psi, tc, _p(out))
    return out


def tdi(freqs, arm_sec, generation, orthogonal, links):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    links = np.ascontiguousarray(links, dtype=np.complex128)
    out = np.zeros((3, freqs.size), dtype=np.complex128)
    lib().oracle_tdi(_p(freqs), freqs.size, arm_sec, int(str(generation) == "2.0"), int(bool(orthogonal)),
                     _p(links), _p(out))
    return out


def whittle(d, h, S, df):
    d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.complex128)
    h = np.ascontiguousarray(np.atleast_2d(h), dtype=np.complex128)
    S = np.ascontiguousarray(np.atleast_2d(S), dtype=np.float64)
    return lib().oracle_whittle(_p(d), _p(h), _p(S), d.shape[0], d.shape[1], df)


def phenomd(theta, freqs, f_ref, f_cut_hz=np.inf, amp_psi=False):
    """IMRPhenomD container (hp, hc, tf) and set-up info; with amp_psi also the
    (2,2) amplitude and unwrapped phase Psi (h22 = A exp(-i Psi)) per frequency."""
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    hp = np.zeros(freqs.size, dtype=np.complex128)
    hc = np.zeros(freqs.size, dtype=np.complex128)
    tf = np.zeros(freqs.size)
    info = np.zeros(18)
    ap = np.zeros((freqs.size, 2)) if amp_psi else None
    lib().oracle_phenomd(_p(theta), _p(freqs), freqs.size, f_ref, float(min(f_cut_hz, 1e300)), _p(hp), _p(hc),
                         _p(tf), _p(info), _p(ap) if amp_psi else None)
    keys = ["M_sec", "fRD", "fDM", "fpeak", "t0", "eta", "gamma1", "gamma2", "gamma3",
            "d0", "d1", "d2", "d3", "d4", "C1Int", "C2Int", "C1MRD", "C2MRD"]
    if amp_psi:
        return hp, hc, tf, dict(zip(keys, info)), ap[:, 0], ap[:, 1]
    return hp, hc, tf, dict(zip(keys, info))


def phenomhm(theta, freqs, f_ref, f_cut_hz=np.inf):
    """IMRPhenomHM container: hp, hc (6, n) complex, tf (6, n), amplitude and
    phase (6, n) (h_lm = A exp(-i Psi)) in mode order HM_MODES, and per mode
    (fRD_lm [Mf], Rholm, amplitude-map inspiral corner [Mf], phase-map
    ringdown corner [Mf])."""
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    n = freqs.size
    hp = np.zeros((6, n), dtype=np.complex128)
    hc = np.zeros((6, n), dtype=np.complex128)
    tf = np.zeros((6, n))
    ap = np.zeros((6, n, 2))
    info = np.zeros((6, 4))
    lib().oracle_phenomhm(_p(theta), _p(freqs), n, f_ref, float(min(f_cut_hz, 1e300)), _p(hp), _p(hc), _p(tf),
                          _p(ap), _p(info))
    return hp, hc, tf, ap[..., 0], ap[..., 1], info


# ------------------------------------------------------------------ grid
def grid(duration, delta_time, minimum_frequency, maximum_frequency):
    """pespace/detector/tdi.py:120-159 semantics, as index arithmetic.

    Returns the masked rfft frequencies plus the first index ``k0``, the rfft
    spacing and the likelihood weight ``delta_frequency = 1/duration``.
    """
    nt = int(duration // delta_time + 1)
    full = np.fft.rfftfreq(nt, delta_time)
    mask = (full >= minimum_frequency) * (full <= maximum_frequency)
    idx = np.nonzero(mask)[0]
    return {
        "time_series_length": nt,
        "full_length": full.size,
        "freqs": full[mask],
        "mask": mask,
        "k0": int(idx[0]) if idx.size else 0,
        "nbins": int(idx.size),
        "f_step": 1.0 / (nt * delta_time),
        "df": 1.0 / duration,
    }


# ------------------------------------------------------------------ PSD
def _s_oms(f, oms, tianqin):
    if tianqin:
        return oms * (2.0 * PI * f / C_SI) ** 2  # noise.py:245
    return oms * (1.0 + (2.0e-3 / f) ** 4) * (2.0 * PI * f / C_SI) ** 2  # noise.py:85-89


def _s_acc(f, acc, tianqin):
    if tianqin:
        return acc * (1.0 + 0.1e-3 / f) / (2 * PI * f * C_SI) ** 2  # noise.py:261-265
    return acc * (1.0 + (0.4e-3 / f) ** 2) * (1.0 + (f / 8e-3) ** 4) / (2 * PI * f * C_SI) ** 2  # noise.py:105-110


def psd(freqs, channels, scaling, tdi_generation, oms_level, acc_level, arm_length_sec, tianqin=False):
    """pespace/detector/noise.py:112-207: analytic PSD per TDI channel."""
    f = np.asarray(freqs, dtype=np.float64)
    S_oms = _s_oms(f, oms_level, tianqin)
    S_acc = _s_acc(f, acc_level, tianqin)
    if scaling:
        sf = (PC_SI / (MRSUN_SI * MTSUN_SI)) ** 2
        S_oms = S_oms * sf
        S_acc = S_acc * sf
    if tdi_generation == "1.5":
        pre = 1.0
    elif tdi_generation == "2.0":
        pre = 4.0 * np.sin(4 * PI * f * arm_length_sec) ** 2
    else:
        raise ValueError(f"The TDI generation {tdi_generation} is unknown")
    L = arm_length_sec
    out = {}
    for c in channels:
        if c in ("X", "Y", "Z"):
            p = 16 * np.sin(2 * PI * f * L) ** 2 * (S_oms + (3 + np.cos(4 * PI * f * L)) * S_acc)
        elif c in ("A", "E"):
            p = 8 * np.sin(2 * PI * f * L) ** 2 * (
                (2 + np.cos(2 * PI * f * L)) * S_oms
                + (6 + 4 * np.cos(2 * PI * f * L) + 2 * np.cos(4 * PI * f * L)) * S_acc)
        elif c == "T":
            p = 32 * np.sin(2 * PI * f * L) ** 2 * np.sin(PI * f * L) ** 2 * (
                S_oms + 4 * np.sin(PI * f * L) ** 2 * S_acc)
        else:
            raise ValueError(f"Unknown TDI channel {c}.")
        out[c] = p * pre
    return out


PSD_PRESETS = {
    # noise.py:268-284
    "LISA_SciRDv1": dict(oms_level=(15.0e-12) ** 2, acc_level=(3.0e-15) ** 2, arm_length_sec=2.5e9 / C_SI),
    "Taiji_TDC": dict(oms_level=(8.0e-12) ** 2, acc_level=(3.0e-15) ** 2, arm_length_sec=3.0e9 / C_SI),
    "Tianqin_GWSpace": dict(oms_level=(1.0e-12) ** 2, acc_level=(1.0e-15) ** 2, arm_length_sec=1.7e8 / C_SI,
                            tianqin=True),
}


def noise_realization(g, psd_by_channel, channels, seed):
    """pespace/detector/tdi.py:896-916: seeded white noise coloured by sqrt(PSD)."""
    rng = np.random.default_rng(seed=seed)
    var = 0.5 / (g["df"]) ** 0.5
    out = {}
    for c in channels:
        re, im = rng.normal(0, var, (2, g["full_length"]))
        re[0] = 0.0
        im[0] = 0.0
        if np.mod(g["time_series_length"], 2) == 0:
            im[-1] = 0.0
            re[-1] = 0.0
        out[c] = (re + 1j * im)[g["mask"]] * np.asarray(psd_by_channel[c]) ** 0.5
    return out


# ------------------------------------------------------------------ batched lnL
class Plan:
    """Keeps the ctypes plan and the arrays it points to alive."""

    def __init__(self, g, detectors, f_ref, cut_factor=0.0, channels=("A", "E", "T"), approximant="IMRPhenomD"):
        self.g = g
        self._keep = []
        dets = (OracleDet * len(detectors))()
        for i, (orbit, gen, data, psd_arr) in enumerate(detectors):
            data = np.ascontiguousarray(data, dtype=np.complex128)
            psd_arr = np.ascontiguousarray(psd_arr, dtype=np.float64)
            self._keep += [data, psd_arr]
            dets[i].orbit = orbit
            dets[i].gen20 = int(str(gen) == "2.0")
            dets[i].data = data.ctypes.data
            dets[i].psd = psd_arr.ctypes.data
        self._dets = dets
        p = OraclePlan()
        p.nbins = g["nbins"]
        p.k0 = g["k0"]
        p.f_step = g["f_step"]
        p.df = g["df"]
        p.f_ref = f_ref
        p.cut_factor = cut_factor
        p.n_det = len(detectors)
        p.chan_mask = sum(1 << "AET".index(c) for c in channels)
        p.dets = ctypes.addressof(dets)
        p.approximant = APPROXIMANTS[approximant]
        self.plan = p

    def lnl(self, theta, grad=False, nthreads=0):
        theta = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        B = theta.shape[0]
        out = np.zeros(B)
        g = np.zeros((B, 11)) if grad else None
        lib().oracle_lnl_batch(ctypes.byref(self.plan), _p(theta), B, _p(out),
                               _p(g) if grad else None, int(nthreads))
        return (out, g) if grad else out

    def fisher(self, theta, nthreads=0):
        """(B, 11, 11) Fisher matrices (fisher.py:27-162) at the rows of theta."""
        theta = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        B = theta.shape[0]
        out = np.zeros((B, 11, 11))
        lib().oracle_fisher_batch(ctypes.byref(self.plan), _p(theta), B, _p(out), int(nthreads))
        return out

    def model_tdi(self, det, theta, orthogonal=True):
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.zeros((3, self.g["nbins"]), dtype=np.complex128)
        lib().oracle_model_tdi(ctypes.byref(self.plan), det, int(orthogonal), _p(theta), _p(out))
        return out
