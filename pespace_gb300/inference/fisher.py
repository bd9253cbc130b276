"""Fisher matrices of the Whittle likelihood (pespace/inference/fisher.py).

``fisher_matrix`` keeps the reference's call (likelihood, fiducial_params,
batch_size) and its definition

    F_ij = 4 df Re sum_{det, c, f} conj(ds_i(f)) ds_j(f) / S_c(f),

computed on the GPU by ``pes_fisher_batch`` at every live bin of the engine's
grid, over its detectors and channels.  FP64 plans use FP64 forward-mode
derivatives.  Mixed plans use the model's structure: PhenomD tangents in
float-float and response tangents in FP32, within 1e-5 of the FP64 matrices
normalised by their diagonal.  The
rows and columns follow the engine's 11-parameter vector (ln Mc, q, chi_1,
chi_2, ln D_L [Mpc], cos iota, lambda, sin beta, psi, phi_c, t_c), not the
fields of the reference's parameter tuple.  ``sample_from_fisher`` and
``wrap_angle_params`` are the reference's host utilities (fisher.py:165-290).
"""

import math

import numpy as np
import torch

from ..waveform.phenomd import theta_from_parameters

PARAMETERS = ("ln_chirp_mass", "mass_ratio", "chi_1", "chi_2", "ln_luminosity_distance", "cos_inclination",
              "ecliptic_longitude", "sin_ecliptic_latitude", "polarization", "reference_phase",
              "coalescence_time")


def _as_theta(fiducial_params):
    """(theta (B, 11), single) from an (11,) / (B, 11) array or a reference-style
    parameter mapping whose entries are scalars or equal-length 1-D arrays."""
    if isinstance(fiducial_params, torch.Tensor):
        th = fiducial_params.detach().to(device="cpu", dtype=torch.float64)
        return (th[None], True) if th.dim() == 1 else (th, False)
    if isinstance(fiducial_params, (np.ndarray, list, tuple)) and not hasattr(fiducial_params, "_fields"):
        th = torch.as_tensor(np.asarray(fiducial_params, dtype=np.float64))
        return (th[None], True) if th.dim() == 1 else (th, False)
    get = fiducial_params.get if isinstance(fiducial_params, dict) else (lambda k, d=None: getattr(fiducial_params, k, d))
    keys = fiducial_params.keys() if isinstance(fiducial_params, dict) else fiducial_params._fields
    values = {k: np.asarray(get(k).detach().cpu() if isinstance(get(k), torch.Tensor) else get(k)) for k in keys}
    shape = np.broadcast_shapes(*(v.shape for v in values.values()))
    if shape == ():
        return torch.as_tensor(theta_from_parameters({k: float(v) for k, v in values.items()}))[None], True
    n = int(np.prod(shape))
    rows = [theta_from_parameters({k: float(np.broadcast_to(v, shape).reshape(-1)[b]) for k, v in values.items()})
            for b in range(n)]
    return torch.as_tensor(np.stack(rows)), False


def fisher_matrix(likelihood, fiducial_params, batch_size=None):
    """Fisher matrix (11, 11) at one parameter set or (B, 11, 11) at a batch.

    likelihood : ``WhittleLikelihood`` (its detectors, PSDs, channels and
        per-sample cut define the sum; the observed data are not used).
    fiducial_params : an (11,) or (B, 11) parameter array, or a mapping with
        the reference's parameter names (scalars, or 1-D arrays of a common
        length for a batch).
    batch_size : samples per GPU call (default: the engine's max_batch).
    """
    if not set(likelihood.channels) <= {"A", "E", "T"}:
        raise ValueError("fisher_matrix requires the independent orthogonal channels ('A', 'E', 'T'), but got the "
                         f"channels {tuple(likelihood.channels)}.")
    theta, single = _as_theta(fiducial_params)
    step = min(int(batch_size), likelihood.max_batch) if batch_size else likelihood.max_batch
    out = torch.cat([likelihood.fisher_matrix(theta[lo:lo + step]) for lo in range(0, theta.shape[0], step)])
    return out[0] if single else out


def sample_from_fisher(fisher, num, rkey_seed=0):
    """``num`` zero-mean samples with covariance ``fisher^{-1}`` (FP64).

    As in the reference: the matrix is first scaled to unit diagonal, the
    scaled matrix is Cholesky-factorised, F' = L L^T, each sample solves
    L^T x' = z for standard normal z, and is scaled back, x = x' / sqrt(diag F);
    no inverse is formed.  The normal variates come from NumPy's generator
    seeded with ``rkey_seed`` (the reference uses JAX's).
    """
    F = np.asarray(fisher.cpu() if isinstance(fisher, torch.Tensor) else fisher, dtype=np.float64)
    scale = np.sqrt(np.diag(F))
    L = np.linalg.cholesky(F / np.outer(scale, scale))
    z = np.random.default_rng(int(rkey_seed)).standard_normal((int(num), F.shape[0]))
    x = np.linalg.solve(L.T, z.T).T
    return x / scale


def _fold(x, lo, hi):
    """Reflect x into [lo, hi] about the boundaries."""
    period = 2.0 * (hi - lo)
    y = np.mod(np.asarray(x, dtype=np.float64) - lo, period)
    return lo + np.where(y > hi - lo, period - y, y)


def wrap_angle_params(samples):
    """Copy of a parameter mapping with the angles in their canonical ranges:
    ecliptic_longitude and reference_phase modulo 2 pi into [0, 2 pi),
    polarization modulo pi into [0, pi), ecliptic_latitude folded into
    [-pi/2, pi/2], inclination folded into [0, pi]; other entries shared."""
    try:
        keys = set(samples.keys())
    except AttributeError as error:
        raise TypeError("samples must be a mapping from parameter names to values") from error
    out = dict(samples) if isinstance(samples, dict) else samples.copy()
    two_pi = 2.0 * math.pi
    if "ecliptic_longitude" in keys:
        out["ecliptic_longitude"] = np.mod(np.asarray(samples["ecliptic_longitude"], dtype=np.float64), two_pi)
    if "reference_phase" in keys:
        out["reference_phase"] = np.mod(np.asarray(samples["reference_phase"], dtype=np.float64), two_pi)
    if "polarization" in keys:
        out["polarization"] = np.mod(np.asarray(samples["polarization"], dtype=np.float64), math.pi)
    if "ecliptic_latitude" in keys:
        out["ecliptic_latitude"] = _fold(samples["ecliptic_latitude"], -0.5 * math.pi, 0.5 * math.pi)
    if "inclination" in keys:
        out["inclination"] = _fold(samples["inclination"], 0.0, math.pi)
    return out
