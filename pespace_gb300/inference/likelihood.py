"""Whittle likelihoods on CUDA.

* ``compute_whittle_likelihood`` replaces ``compute_whittle_likelihood_ti``
  (pespace/inference/likelihood_ti.py:17-69) and ``noise_weighted_inner_product``
  replaces the JAX kernel (likelihood_jax.py:21-42).
* ``LikelihoodBilbyInterface`` keeps ``LikelihoodBilbyInterfaceTaichi``'s
  constructor and ``log_likelihood(parameters)`` (interface_bilby.py:31-116),
  one sample at a time through the plugin kernels.
* ``WhittleLikelihood`` is the batched engine: one plan, many samples per call,
  lnL and its 11-parameter gradient (behind ``torch.autograd``).
"""

import ctypes
from collections import namedtuple

import numpy as np
import torch

from .. import _lib
from ..waveform.phenomd import IMRPhenomD, theta_from_parameters


def _rows(data, labels, channels):
    idx = [labels.index(c) for c in channels]
    return data[idx].contiguous()


def noise_weighted_inner_product(observed_data, response_data, psd, df):
    """-2 df sum |d - h|^2 / S over (C, N) (or (N,)) CUDA tensors; returns a float."""
    d = torch.as_tensor(observed_data, dtype=torch.complex128, device="cuda")
    h = torch.as_tensor(response_data, dtype=torch.complex128, device="cuda")
    s = torch.as_tensor(psd, dtype=torch.float64, device="cuda")
    if d.dim() == 1:
        d, h, s = d[None], h[None], s[None]
    d, h, s = d.contiguous(), h.contiguous(), s.contiguous()
    if not (d.shape == h.shape == s.shape):
        raise ValueError(f"shape mismatch: data {tuple(d.shape)}, response {tuple(h.shape)}, psd {tuple(s.shape)}")
    C, N = d.shape
    lib = _lib.load()
    ws = torch.empty(int(lib.pes_whittle_workspace_len(N)), dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(lib.pes_whittle_lnl(_lib.ptr(d), _lib.ptr(h), _lib.ptr(s), C, N, float(df), _lib.ptr(ws),
                                   ws.numel(), _lib.ptr(out), _lib.stream_handle()))
    return float(out.item())


def compute_whittle_likelihood(channels, observed_data, response_data, psd, df, labels=("A", "E", "T")):
    """likelihood_ti.py:17-69 over the listed channels of (C, N) tensors."""
    return noise_weighted_inner_product(_rows(observed_data, labels, channels), _rows(response_data, labels, channels),
                                        _rows(psd, labels, channels), df)


# the reference's name for the same call (likelihood_ti.py:17)
compute_whittle_likelihood_ti = compute_whittle_likelihood


class LikelihoodBilbyInterface:
    """interface_bilby.py:21-116 without the bilby base class (bilby is optional)."""

    def __init__(self, waveform, detector, channels):
        self.waveform = waveform
        if not isinstance(detector, tuple):
            detector = (detector,)
        self.detector = detector
        unsupported = [c for c in channels if c not in ("A", "E", "T")]
        if any(unsupported):
            raise ValueError("The likelihood compution only support TDI channels of ('A','E','T'). "
                             f"{unsupported} are not supported currently.")
        self.channels = tuple(channels)
        self.parameters = {}

    def log_likelihood(self, parameters=None):
        parameters = self.parameters if parameters is None else parameters
        self.waveform.update_waveform(parameters)
        logl = 0.0
        for det in self.detector:
            det.update_detector_response(self.waveform.waveform_container, parameters["ecliptic_longitude"],
                                         parameters["ecliptic_latitude"], parameters["polarization"],
                                         parameters["coalescence_time"])
            logl += compute_whittle_likelihood(self.channels, det.tdi_data.fd_data, det.tdi_response,
                                               det.tdi_data.fd_noise_power_density,
                                               det.tdi_data.data_info.delta_frequency,
                                               labels=det.tdi_combination.labels)
        return logl


class WhittleLikelihood:
    """Batched lnL / lnL+gradient over parameter samples on one GPU.

    Parameters
    ----------
    detector : InterferometerAntenna or tuple of them (same frequency grid,
        orthogonal A/E/T combination).  Their ``tdi_data`` must hold
        ``fd_data`` and ``fd_noise_power_density``.
    channels : subset of ("A", "E", "T").
    precision : "fp64" (dense FP64, every bin) or "mixed" (float-float sparse
        grid, FP32 dense bulk, the samples near the accuracy target
        re-evaluated).
    cut_factor : per-sample model cutoff in units of the ringdown frequency
        (the largest of the modes' for IMRPhenomHM; 0 keeps the model's own
        Mf = 0.2 cut only).
    approximant : "IMRPhenomD" (the (2,2) mode) or "IMRPhenomHM" (modes
        (2,2), (2,1), (3,3), (3,2), (4,4), (4,3); lnL, gradient and Fisher
        matrices from FP64 plans, lnL and Fisher matrices from mixed plans).
    """

    APPROXIMANTS = {"IMRPhenomD": _lib.APPROX_PHENOMD, "IMRPhenomHM": _lib.APPROX_PHENOMHM}

    def __init__(self, detector, channels=("A", "E", "T"), precision="fp64", reference_frequency=None,
                 cut_factor=0.0, max_batch=1024, n_sparse=1024, approximant="IMRPhenomD"):
        if not isinstance(detector, tuple):
            detector = (detector,)
        if len(detector) > _lib.MAX_DETECTORS:
            raise ValueError(f"at most {_lib.MAX_DETECTORS} detectors")
        unsupported = [c for c in channels if c not in ("A", "E", "T")]
        if any(unsupported):
            raise ValueError(f"The likelihood computation only supports orthogonal channels ('A', 'E', 'T'). "
                             f"{unsupported} are not supported currently.")
        info0 = detector[0].tdi_data.data_info
        for det in detector:
            if det.tdi_combination.labels != ("A", "E", "T"):
                raise ValueError(f"detector {det.name} must use the orthogonal (A, E, T) combination")
            info = det.tdi_data.data_info
            if (info.frequency_series_length, info.first_index, info.frequency_step) != (
                    info0.frequency_series_length, info0.first_index, info0.frequency_step):
                raise ValueError("all detectors must share one frequency grid")
            if det.tdi_data.fd_data is None or det.tdi_data.fd_noise_power_density is None:
                raise ValueError(f"fd_data and fd_noise_power_density must be set for detector={det.name}")
        self.detector = detector
        self.channels = tuple(channels)
        self.precision = precision
        # likelihood_jax.py:119-127: waveform parameters, then the response's
        self.likelihood_param_type = namedtuple(
            "LikelihoodParams", (*IMRPhenomD.required_params, "ecliptic_longitude", "ecliptic_latitude",
                                 "polarization", "coalescence_time"))
        self.max_batch = int(max_batch)
        desc = _lib.PesPlanDesc()
        desc.nbins = info0.frequency_series_length
        desc.k0 = info0.first_index
        desc.f_step = info0.frequency_step
        desc.df = info0.delta_frequency
        desc.f_ref = float(reference_frequency if reference_frequency is not None else info0.minimum_frequency)
        desc.cut_factor = float(cut_factor)
        desc.n_det = len(detector)
        desc.chan_mask = sum(1 << "AET".index(c) for c in self.channels)
        desc.precision = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}[precision]
        desc.n_sparse = int(n_sparse)
        desc.max_batch = self.max_batch
        if approximant not in self.APPROXIMANTS:
            raise ValueError(f"unknown approximant {approximant}; available: {sorted(self.APPROXIMANTS)}")
        desc.approximant = self.APPROXIMANTS[approximant]
        self.approximant = approximant
        for i, det in enumerate(detector):
            desc.det[i].orbit = det.orbit_model.to_c()
            desc.det[i].generation = det.tdi_combination.generation_code
        self.desc = desc
        lib = _lib.load()
        handle = ctypes.c_void_p()
        _lib.check(lib.pes_plan_create(ctypes.byref(desc), ctypes.byref(handle)))
        self._plan = handle
        for i, det in enumerate(detector):
            data = det.tdi_data.fd_data.to(torch.complex128).contiguous()
            psd = det.tdi_data.fd_noise_power_density.to(torch.float64).contiguous()
            _lib.check(lib.pes_plan_set_data(self._plan, i, _lib.ptr(data), _lib.ptr(psd), _lib.stream_handle()))
        self.last_status = None

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                _lib.load().pes_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    def _prep(self, theta):
        theta = torch.as_tensor(theta, dtype=torch.float64, device="cuda")
        if theta.dim() == 1:
            theta = theta[None]
        if theta.shape[-1] != 11:
            raise ValueError(f"theta must have 11 columns, got {tuple(theta.shape)}")
        return theta.contiguous()

    def log_likelihood_batch(self, theta):
        """lnL for a (B, 11) parameter tensor; returns a (B,) CUDA tensor."""
        theta = self._prep(theta)
        B = theta.shape[0]
        out = torch.empty(B, dtype=torch.float64, device="cuda")
        status = torch.empty(B, dtype=torch.int32, device="cuda")
        for lo in range(0, B, self.max_batch):
            hi = min(B, lo + self.max_batch)
            _lib.check(_lib.load().pes_lnl_batch(self._plan, _lib.ptr(theta[lo:hi]), hi - lo, _lib.ptr(out[lo:hi]),
                                                 _lib.ptr(status[lo:hi]), _lib.stream_handle()))
        self.last_status = status
        return out

    def log_likelihood_and_grad(self, theta):
        """(lnL (B,), dlnL/dtheta (B, 11)) for a (B, 11) parameter tensor."""
        theta = self._prep(theta)
        B = theta.shape[0]
        out = torch.empty(B, dtype=torch.float64, device="cuda")
        grad = torch.empty((B, 11), dtype=torch.float64, device="cuda")
        status = torch.empty(B, dtype=torch.int32, device="cuda")
        for lo in range(0, B, self.max_batch):
            hi = min(B, lo + self.max_batch)
            _lib.check(_lib.load().pes_lnl_grad_batch(self._plan, _lib.ptr(theta[lo:hi]), hi - lo,
                                                      _lib.ptr(out[lo:hi]), _lib.ptr(grad[lo:hi]),
                                                      _lib.ptr(status[lo:hi]), _lib.stream_handle()))
        self.last_status = status
        return out, grad

    @property
    def refine_all(self):
        """Mixed plans: True when every sample's dense range is re-evaluated
        (``PES_OPT_REFINE_ALL``: in float-float from its splines, or exactly
        where the splines' error estimate exceeds the target), False (the
        default) when only the samples whose error estimates approach the
        accuracy target are."""
        v = ctypes.c_int64()
        _lib.check(_lib.load().pes_plan_get_option(self._plan, _lib.PES_OPT_REFINE_ALL, ctypes.byref(v)))
        return bool(v.value)

    @refine_all.setter
    def refine_all(self, on):
        _lib.check(_lib.load().pes_plan_set_option(self._plan, _lib.PES_OPT_REFINE_ALL, int(bool(on))))

    @property
    def launch_options(self):
        """The plan's launch options: {"dense_stage": 0 | 1, "sample_threads": n}."""
        from .autotune import OPTIONS, get_option

        return {name: get_option(self, name) for name in OPTIONS}

    def autotune(self, theta, grad=True, reps=5, candidates=None):
        """Time the plan's launch options on the batch ``theta`` and keep the
        fastest (``pespace_gb300.inference.autotune.autotune``)."""
        from .autotune import autotune

        return autotune(self, theta, grad=grad, reps=reps, candidates=candidates)

    def fisher_matrix(self, theta):
        """(B, 11, 11) Fisher matrices at the rows of a (B, 11) parameter tensor
        (fisher.py:27-162 over this engine's detectors, channels and per-sample
        cut).  FP64 plans use FP64 forward derivatives; mixed plans use
        float-float values and tangents for the waveform and FP32 duals for
        the response (within 1e-5 of the FP64 matrices, normalised by the
        diagonal)."""
        theta = self._prep(theta)
        B = theta.shape[0]
        out = torch.empty((B, 11, 11), dtype=torch.float64, device="cuda")
        status = torch.empty(B, dtype=torch.int32, device="cuda")
        for lo in range(0, B, self.max_batch):
            hi = min(B, lo + self.max_batch)
            _lib.check(_lib.load().pes_fisher_batch(self._plan, _lib.ptr(theta[lo:hi]), hi - lo, _lib.ptr(out[lo:hi]),
                                                    _lib.ptr(status[lo:hi]), _lib.stream_handle()))
        self.last_status = status
        return out

    def last_work(self, batch):
        """Work units of the last call on ``batch`` samples (the last chunk when the
        call was split at max_batch): dict with the bins through the FP32 dense
        stage, the bins evaluated directly in FP64, the sparse-node evaluations,
        the samples in the parameter domain, and the samples whose dense range
        was re-evaluated in float-float and exactly."""
        out = (ctypes.c_int64 * 6)()
        _lib.check(_lib.load().pes_plan_work(self._plan, min(int(batch), self.max_batch), out,
                                             _lib.stream_handle()))
        return {"dense_bins": out[0], "fp64_bins": out[1], "sparse_nodes": out[2], "samples": out[3],
                "refined_ff": out[4], "refined_exact": out[5]}

    def log_likelihood(self, params):
        """likelihood_jax.py:207-260 call: a ``likelihood_param_type`` namedtuple
        (or a dict with the same names).  Scalar fields give a float; 1-D array
        fields of a common length (what a vectorised sampler passes) give a
        (B,) CUDA tensor evaluated in one batched call."""
        from .fisher import _as_theta

        theta, single = _as_theta(params)
        out = self.log_likelihood_batch(theta)
        return float(out[0].item()) if single else out

    def model_tdi(self, theta, det=0, orthogonal=True):
        """Dense A/E/T model of one detector (parity / debugging)."""
        theta = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(11))
        out = torch.empty((3, int(self.desc.nbins)), dtype=torch.complex128, device="cuda")
        _lib.check(_lib.load().pes_plan_model_tdi(self._plan, det, int(orthogonal), _lib.ptr(theta), _lib.ptr(out),
                                                  _lib.stream_handle()))
        return out


class WhittleLikelihoodCuda(WhittleLikelihood):
    """``WhittleLikelihoodJax`` (likelihood_jax.py:45-260) with the reference's
    constructor ``(waveform, detector, channels)``.

    The waveform must be this package's ``IMRPhenomD``, and its frequencies
    must equal every detector's frequency samples (the reference's checks,
    likelihood_jax.py:84-112).  Its reference frequency becomes the plan's.
    ``likelihood_param_type`` is built from the waveform's ``required_params``
    and the response's four parameters.  ``log_likelihood(params)`` takes that
    tuple.  The GPU options (``precision``, ``cut_factor``, ``max_batch``,
    ``n_sparse``) are keyword-only.
    """

    def __init__(self, waveform, detector, channels, *, precision="fp64", cut_factor=0.0, max_batch=1024,
                 n_sparse=1024):
        if not isinstance(waveform, IMRPhenomD):
            raise TypeError("WhittleLikelihoodCuda requires the waveform to be an IMRPhenomD instance, but got "
                            f"{type(waveform).__name__}.")
        dets = detector if isinstance(detector, tuple) else (detector,)
        for det in dets:
            if det.backend != "cuda":
                raise ValueError("WhittleLikelihoodCuda requires all detectors configured with backend='cuda', "
                                 f"but got backend={det.backend} for detector={det.name}.")
            fs = det.tdi_data.frequency_samples
            if fs is None or fs.shape != waveform.frequencies.shape or not torch.equal(
                    fs.to(waveform.frequencies.device), waveform.frequencies):
                raise ValueError("The waveform frequencies should match the frequency samples of the TDI data "
                                 f"for detector={det.name}.")
        super().__init__(dets, channels, precision=precision, reference_frequency=waveform.reference_frequency,
                         cut_factor=cut_factor, max_batch=max_batch, n_sparse=n_sparse)
        self.waveform = waveform


class CapturedStep:
    """One batched lnL (+ gradient) call of an engine captured in a CUDA graph.

    The graph is recorded once on fixed device buffers (``theta``, ``lnl``,
    ``grad``, ``status``); ``__call__`` copies new parameters into ``theta``
    and replays it, which removes the per-launch host cost of the kernels and
    event waits of a call.  A batch larger than the engine's ``max_batch``
    is captured as consecutive calls of ``max_batch`` samples.  The engine's
    measurement hooks must be off while capturing.
    """

    def __init__(self, engine, batch, grad=True):
        if batch < 1:
            raise ValueError(f"batch must be at least 1, got {batch}")
        self.engine, self.batch, self.with_grad = engine, int(batch), bool(grad)
        dev = torch.device("cuda")
        self.theta = torch.zeros((batch, 11), dtype=torch.float64, device=dev)
        self.lnl = torch.empty(batch, dtype=torch.float64, device=dev)
        self.grad = torch.empty((batch, 11), dtype=torch.float64, device=dev) if grad else None
        self.status = torch.empty(batch, dtype=torch.int32, device=dev)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self._launch()  # warm-up outside the capture
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch()

    def _launch(self):
        lib = _lib.load()
        for lo in range(0, self.batch, self.engine.max_batch):
            hi = min(self.batch, lo + self.engine.max_batch)
            th, ln, st = self.theta[lo:hi], self.lnl[lo:hi], self.status[lo:hi]
            if self.with_grad:
                rc = lib.pes_lnl_grad_batch(self.engine._plan, _lib.ptr(th), hi - lo, _lib.ptr(ln),
                                            _lib.ptr(self.grad[lo:hi]), _lib.ptr(st), _lib.stream_handle())
            else:
                rc = lib.pes_lnl_batch(self.engine._plan, _lib.ptr(th), hi - lo, _lib.ptr(ln), _lib.ptr(st),
                                       _lib.stream_handle())
            _lib.check(rc)

    def __call__(self, theta):
        """Replay on new parameters (B, 11); returns lnL (and the gradient) views of the graph's buffers."""
        self.theta.copy_(torch.as_tensor(theta, dtype=torch.float64, device="cuda").reshape(self.batch, 11))
        self.graph.replay()
        return (self.lnl, self.grad) if self.with_grad else self.lnl


class _LogLikelihoodFn(torch.autograd.Function):
    """lnL(theta) with the gradient from the plan's adjoint kernels.

    The forward pass runs the lnL-only call and keeps nothing but the
    parameters.  The backward pass runs the lnL+gradient call, which
    recomputes the sparse-grid waveform and transfer, the splines and the
    dense stage (accumulating the interval moments), then the transposed
    spline solve and the backward node pass: no dense residuals are stored
    between the two passes."""

    @staticmethod
    def forward(ctx, theta, engine):
        ctx.engine = engine
        ctx.save_for_backward(theta)
        return engine.log_likelihood_batch(theta)

    @staticmethod
    def backward(ctx, g):
        (theta,) = ctx.saved_tensors
        _, grad = ctx.engine.log_likelihood_and_grad(theta)
        return (g[:, None] * grad).reshape(theta.shape), None


def log_likelihood(theta, engine):
    """Differentiable batched lnL: ``log_likelihood(theta, engine).sum().backward()``."""
    return _LogLikelihoodFn.apply(theta, engine)
