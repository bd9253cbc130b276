"""TDI data container and FD TDI combination (pespace/detector/tdi.py) on CUDA.

Storage is channel-major: ``fd_data`` is a (C, N) complex128 CUDA tensor and
``fd_noise_power_density`` a (C, N) float64 CUDA tensor, C = len(channels).
"""

import warnings
from abc import ABC, abstractmethod
from collections import namedtuple
from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _lib
from .noise import FrequencyDomainNoiseModel, available_noise_models


@dataclass(frozen=True)
class DataInformation:
    """tdi.py:64-159: the dense frequency grid of a dataset.

    ``frequency_samples_array`` = rfftfreq(int(duration // delta_time + 1),
    delta_time) masked to [minimum_frequency, maximum_frequency]; its spacing is
    1/(Nt dt).  The likelihood weight is ``delta_frequency`` = 1/duration.
    """

    channels: tuple
    duration: float
    delta_time: float
    start_time: float
    minimum_frequency: float
    maximum_frequency: float
    sampling_frequency: float = field(init=False)
    delta_frequency: float = field(init=False)
    time_series_length: int = field(init=False)
    full_frequency_series_length: int = field(init=False)
    frequency_mask_array: np.ndarray = field(init=False)
    frequency_samples_array: np.ndarray = field(init=False)
    frequency_series_length: int = field(init=False)
    first_index: int = field(init=False)
    frequency_step: float = field(init=False)

    def __post_init__(self):
        nt = int(self.duration // self.delta_time + 1)
        full = np.fft.rfftfreq(nt, self.delta_time)
        mask = (full >= self.minimum_frequency) * (full <= self.maximum_frequency)
        idx = np.nonzero(mask)[0]
        for k, v in dict(
            sampling_frequency=1 / self.delta_time,
            delta_frequency=1 / self.duration,
            time_series_length=nt,
            full_frequency_series_length=int(full.size),
            frequency_mask_array=mask,
            frequency_samples_array=full[mask],
            frequency_series_length=int(idx.size),
            first_index=int(idx[0]) if idx.size else 0,
            frequency_step=1.0 / (nt * self.delta_time),
        ).items():
            object.__setattr__(self, k, v)

    @property
    def time_samples_array(self):
        return np.arange(self.time_series_length) * self.delta_time + self.start_time


def fd_from_td(td_array, info, window=None):
    """tdi.py:661-726 (set_fd_data_from_td): per channel, rfft of the windowed
    series divided by the sampling frequency, cropped to the frequency mask.

    td_array : (C, time_series_length) real array; info : DataInformation;
    window : None (no window), an array of time_series_length weights, or a
        ``scipy.signal.get_window`` specification.  Host NumPy, like the
        reference (a one-time set-up step).
    """
    n = info.time_series_length
    if window is None:
        weight = np.ones(n)
    elif isinstance(window, np.ndarray):
        weight = window
    else:
        from scipy import signal

        weight = signal.get_window(window, n)
    out = [np.fft.rfft(np.asarray(row, dtype=np.float64) * weight) / info.sampling_frequency for row in td_array]
    return np.stack([row[info.frequency_mask_array] for row in out]).astype(np.complex128)


def fd_noise_realization_array(info, psd, seed=None):
    """tdi.py:896-916 on the host: per channel, one draw of
    ``default_rng(seed).normal(0, 0.5 / sqrt(delta_frequency), (2, full length))``
    as real and imaginary parts, zero at DC (and at Nyquist for an even number
    of time samples), cropped to the frequency mask and scaled by sqrt(PSD).
    info : DataInformation; psd : (C, frequency_series_length) array.
    Returns a (C, frequency_series_length) complex128 array."""
    rng = np.random.default_rng(seed=seed)
    var = 0.5 / (info.delta_frequency) ** 0.5
    psd = np.asarray(psd, dtype=np.float64)
    out = []
    for c_i, _ in enumerate(info.channels):
        re, im = rng.normal(0, var, (2, info.full_frequency_series_length))
        re[0] = 0.0
        im[0] = 0.0
        if np.mod(info.time_series_length, 2) == 0:
            im[-1] = 0.0
            re[-1] = 0.0
        out.append((re + 1j * im)[info.frequency_mask_array] * psd[c_i] ** 0.5)
    return np.stack(out)


# data_info keys of the HDF5 file, in the reference's DataInformation field order (tdi.py:64-101)
_INFO_KEYS = ("channels", "duration", "delta_time", "start_time", "minimum_frequency", "maximum_frequency",
              "sampling_frequency", "delta_frequency", "time_series_length", "time_samples_array",
              "full_frequency_series_length", "full_frequency_samples_array", "frequency_mask_array",
              "frequency_samples_array", "frequency_series_length")


def _h5py():
    try:
        import h5py
    except ImportError as error:
        raise ImportError("HDF5 save/recover needs h5py, which is not installed") from error
    return h5py


def _as_str(x):
    x = x[()] if isinstance(x, np.ndarray) and x.ndim == 0 else x
    return x.decode("utf-8") if isinstance(x, (bytes, np.bytes_)) else str(x)


def _info_values(info):
    values = {k: getattr(info, k) for k in _INFO_KEYS if k not in ("time_samples_array",
                                                                    "full_frequency_samples_array")}
    values["time_samples_array"] = info.time_samples_array
    values["full_frequency_samples_array"] = np.fft.rfftfreq(info.time_series_length, info.delta_time)
    return values


def _hdf5_write(filename, scaling, backend, info, arrays):
    """tdi.py:1022-1097 layout: class_attrs/{scaling, backend, _np_fp, _np_cp},
    data_info/<field>, tdi_data/{td_data, fd_data}/<chan>,
    noise_data/fd_noise_power_density/<chan>.  ``arrays``: {key: (C, n) array or None}."""
    h5py = _h5py()
    string = h5py.string_dtype(encoding="utf-8")
    with h5py.File(filename, "x") as file:
        file.create_dataset("class_attrs/scaling", data=np.array(scaling))
        file.create_dataset("class_attrs/backend", data=np.array(backend, dtype=string))
        file.create_dataset("class_attrs/_np_fp", data=np.array("float64", dtype=string))
        file.create_dataset("class_attrs/_np_cp", data=np.array("complex128", dtype=string))
        values = _info_values(info)
        for key in _INFO_KEYS:
            if key == "channels":
                file.create_dataset(f"data_info/{key}", data=np.array(values[key], dtype=string))
            else:
                file.create_dataset(f"data_info/{key}", data=np.array(values[key]))
        for group, keys in (("tdi_data", ("td_data", "fd_data")), ("noise_data", ("fd_noise_power_density",))):
            for key in keys:
                data = arrays.get(key)
                if data is not None:
                    for c_i, chan in enumerate(info.channels):
                        file.create_dataset(f"{group}/{key}/{chan}", data=np.asarray(data[c_i]))


def _hdf5_read(filename):
    """tdi.py:1099-1292: (scaling, DataInformation, {key: (C, n) array}) with
    the reference's checks of the stored precision and derived quantities
    (AssertionError on a mismatch).  The stored backend is not used: the
    data are recovered onto this package's CUDA backend."""
    h5py = _h5py()
    with h5py.File(filename, "r") as file:
        scaling = bool(file["class_attrs/scaling"][()])
        fp, cp = _as_str(file["class_attrs/_np_fp"][()]), _as_str(file["class_attrs/_np_cp"][()])
        assert fp == "float64" and cp == "complex128", (
            f"Failed to recover TDIChannelData from file {filename}.\nThe numerical precision of stored data "
            f"does not match the settings of the current environment.\nThe stored data have _np_fp={fp}, and "
            f"_np_cp={cp}.\nWhile TDIChannelData in the current environment is initialized with "
            "_np_fp=float64, and _np_cp=complex128.")
        channels = tuple(_as_str(c) for c in file["data_info/channels"][()])
        args = [float(file[f"data_info/{k}"][()]) for k in ("duration", "delta_time", "start_time",
                                                            "minimum_frequency", "maximum_frequency")]
        info = DataInformation(channels, *args)
        values = _info_values(info)
        for key in _INFO_KEYS[6:]:
            stored = file[f"data_info/{key}"][()]
            same = np.array_equal(values[key], stored) if np.ndim(stored) else values[key] == stored
            assert same, (f"Failed to recover TDIChannelData from file {filename}, the `{key}` is different "
                          "from the stored value.")
        arrays = {}
        for group, keys in (("tdi_data", ("td_data", "fd_data")), ("noise_data", ("fd_noise_power_density",))):
            if group not in file:
                continue
            for key in keys:
                if key in file[group]:
                    arrays[key] = np.stack([np.asarray(file[f"{group}/{key}/{chan}"][()]) for chan in channels])
    return scaling, info, arrays


class TDIChannelData:
    """tdi.py:162-1376 with CUDA tensors: ``td_data`` (C, time_series_length)
    float64, ``fd_data`` (C, frequency_series_length) complex128; the
    wavelet domain and the conversions the reference leaves unimplemented
    raise NotImplementedError as there."""

    def __init__(self, scaling=False, backend="cuda"):
        if backend != "cuda":
            raise ValueError(f"Invalid backend: {backend}")
        self.scaling = scaling
        self.backend = backend
        self._reset()

    def _reset(self):
        self.time_samples = None
        self.frequency_samples = None
        self.td_data = None
        self.fd_data = None
        self.fd_noise_power_density = None
        self._data_info = None
        self._reset_flag = False

    @property
    def data_info(self):
        return self._data_info

    def set_data_info(self, channels, duration, delta_time, start_time, minimum_frequency, maximum_frequency):
        if self._reset_flag:
            warnings.warn("You are setting `data_info`, but you have set TDI data of current instance previously.")
        self._data_info = DataInformation(tuple(channels), duration, delta_time, start_time, minimum_frequency,
                                          maximum_frequency)

    def set_fd_data_from_zero(self, channels, duration, delta_time, start_time=0.0, minimum_frequency=1e-5,
                              maximum_frequency=0.1):
        if self._reset_flag:
            warnings.warn("You are setting `fd_data` with zero value; the instance is reset.")
            self._reset()
        self.set_data_info(channels, duration, delta_time, start_time, minimum_frequency, maximum_frequency)
        n = self.data_info.frequency_series_length
        self.frequency_samples = torch.as_tensor(self.data_info.frequency_samples_array, dtype=torch.float64,
                                                 device="cuda")
        self.fd_data = torch.zeros((len(channels), n), dtype=torch.complex128, device="cuda")
        self._reset_flag = True

    def set_fd_data_from_input(self, channels, duration, delta_time, tdi_data_array, start_time=0.0,
                               minimum_frequency=1e-5, maximum_frequency=0.1):
        self.set_fd_data_from_zero(channels, duration, delta_time, start_time, minimum_frequency, maximum_frequency)
        arr = torch.as_tensor(np.asarray(tdi_data_array), dtype=torch.complex128, device="cuda")
        if tuple(arr.shape) != tuple(self.fd_data.shape):
            raise ValueError(f"tdi_data_array must have shape {tuple(self.fd_data.shape)}, got {tuple(arr.shape)}; "
                             "crop it with `data_info.frequency_mask_array` first")
        self.fd_data.copy_(arr)

    def set_td_data_from_input(self, channels, duration, delta_time, tdi_data_array, start_time=0.0,
                               minimum_frequency=1e-5, maximum_frequency=0.1):
        """tdi.py:330-414: time-domain data from a (len(channels), time_series_length) array."""
        if self._reset_flag:
            warnings.warn("You are setting `td_data` with input array, but you have set TDI data of current "
                          "instance previously; the instance is reset.")
            self._reset()
        self.set_data_info(channels, duration, delta_time, start_time, minimum_frequency, maximum_frequency)
        arr = np.asarray(tdi_data_array, dtype=np.float64)
        channels_num, samples_num = arr.shape
        if len(channels) != channels_num:
            raise ValueError(f"You set channels with {channels}, while the length of first dimension "
                             f"of input tdi_data_array is {channels_num}.")
        if self.data_info.time_series_length != samples_num:
            raise ValueError(f"The length of second dimension of input array is {samples_num}. It is different "
                             f"with the `time_series_length={self.data_info.time_series_length}` which is set "
                             "according to the duration and delta_time by `int(duration//delta_time + 1)`.")
        self.time_samples = torch.as_tensor(self.data_info.time_samples_array, dtype=torch.float64, device="cuda")
        self.td_data = torch.as_tensor(arr, device="cuda")
        self._reset_flag = True

    def set_td_data_from_zero(self, channels, duration, delta_time, start_time=0.0, minimum_frequency=1e-5,
                              maximum_frequency=0.1):
        """tdi.py:521-583: time-domain data of zeros."""
        if self._reset_flag:
            warnings.warn("You are setting `td_data` with zero value; the instance is reset.")
            self._reset()
        self.set_data_info(channels, duration, delta_time, start_time, minimum_frequency, maximum_frequency)
        self.time_samples = torch.as_tensor(self.data_info.time_samples_array, dtype=torch.float64, device="cuda")
        self.td_data = torch.zeros((len(channels), self.data_info.time_series_length), dtype=torch.float64,
                                   device="cuda")
        self._reset_flag = True

    def set_fd_data_from_td(self, window=None):
        """tdi.py:661-726: ``fd_data`` from ``td_data`` (``fd_from_td``); the start
        time is not applied as a phase shift, as in the reference."""
        if self.td_data is None or self.fd_data is not None:
            raise ValueError("Fourier transform cannot be executed since the `td_data` is not set or "
                             "`fd_data` has been set previously.")
        arr = fd_from_td(self.td_data.cpu().numpy(), self.data_info, window)
        self.frequency_samples = torch.as_tensor(self.data_info.frequency_samples_array, dtype=torch.float64,
                                                 device="cuda")
        self.fd_data = torch.as_tensor(arr, device="cuda")

    def set_td_data_from_fd(self, window=None):
        raise NotImplementedError()

    def set_wd_data_from_zero(self):
        raise NotImplementedError()

    def set_wd_data_from_td(self):
        raise NotImplementedError()

    def set_wd_data_from_fd(self):
        raise NotImplementedError()

    def set_fd_noise_power_density_from_td_data(self):
        raise NotImplementedError()

    def get_td_noise_realization(self):
        raise NotImplementedError()

    def set_fd_noise_power_density_from_model(self, noise_model, **model_kwargs):
        if isinstance(noise_model, str):
            if noise_model not in available_noise_models:
                raise ValueError(f"{noise_model} is not an implemented noise model. \n"
                                 f"Current available noise models include {[*available_noise_models.keys()]}.")
            psd = available_noise_models[noise_model]
        elif isinstance(noise_model, FrequencyDomainNoiseModel):
            psd = noise_model
        else:
            raise TypeError(f"unsupported noise model {type(noise_model).__name__}")
        if self.data_info is None:
            raise ValueError("The `data_info` has not yet set.")
        if self.fd_noise_power_density is not None:
            warnings.warn("`fd_noise_power_density` has been set previously; it is replaced.")
        d = psd(self.data_info.frequency_samples_array, self.data_info.channels, self.scaling, **model_kwargs)
        arr = np.stack([np.asarray(d[c], dtype=np.float64) for c in self.data_info.channels])
        self.fd_noise_power_density = torch.as_tensor(arr, device="cuda")

    def get_fd_noise_realization(self, seed=None, output_type="cuda"):
        """tdi.py:896-916: seeded white noise coloured by sqrt(PSD) (host RNG)."""
        if self.fd_noise_power_density is None:
            raise ValueError("Setting `fd_noise_power_density` before generating noise realization.")
        info = self.data_info
        arr = fd_noise_realization_array(info, self.fd_noise_power_density.cpu().numpy(), seed)
        if output_type == "numpy":
            return namedtuple("DataContent", info.channels)(*arr)
        if output_type == "cuda":
            return torch.as_tensor(arr, dtype=torch.complex128, device="cuda")
        raise ValueError(f"Unknown output_type: {output_type}")

    def save_to_file(self, filename):
        """tdi.py:1022-1097: the instance's data as an HDF5 file (h5py; the
        file must not exist)."""
        _hdf5_write(filename, self.scaling, self.backend, self.data_info,
                    {"td_data": None if self.td_data is None else self.td_data.cpu().numpy(),
                     "fd_data": None if self.fd_data is None else self.fd_data.cpu().numpy(),
                     "fd_noise_power_density": None if self.fd_noise_power_density is None
                     else self.fd_noise_power_density.cpu().numpy()})

    @staticmethod
    def recover_from_file(filename):
        """tdi.py:1099-1292: a TDIChannelData from a file written by
        ``save_to_file`` (here or by the reference), on the CUDA backend."""
        scaling, info, arrays = _hdf5_read(filename)
        ret = TDIChannelData(scaling=scaling)
        ret._data_info = info
        if "td_data" in arrays:
            ret.time_samples = torch.as_tensor(info.time_samples_array, dtype=torch.float64, device="cuda")
            ret.td_data = torch.as_tensor(arrays["td_data"], dtype=torch.float64, device="cuda")
        if "fd_data" in arrays:
            ret.frequency_samples = torch.as_tensor(info.frequency_samples_array, dtype=torch.float64,
                                                    device="cuda")
            ret.fd_data = torch.as_tensor(arrays["fd_data"], dtype=torch.complex128, device="cuda")
        if "fd_noise_power_density" in arrays:
            ret.fd_noise_power_density = torch.as_tensor(arrays["fd_noise_power_density"], dtype=torch.float64,
                                                         device="cuda")
        ret._reset_flag = True
        return ret

    def add_into_td_data(self):
        raise NotImplementedError()

    def add_into_wd_data(self):
        raise NotImplementedError()

    @property
    def wd_data_numpy(self):
        return None  # no wavelet-domain data (not implemented, as in the reference)

    def add_into_fd_data(self, input):
        arr = input if torch.is_tensor(input) else torch.as_tensor(np.stack(list(input)), device="cuda")
        if tuple(arr.shape) != tuple(self.fd_data.shape):
            raise ValueError("Cannot add the input into the `fd_data`: shape differs from the TDI data")
        self.fd_data += arr.to(self.fd_data.dtype)

    @property
    def td_data_numpy(self):
        if self.td_data is None:
            return None
        return namedtuple("DataContent", self.data_info.channels)(*self.td_data.cpu().numpy())

    @property
    def fd_data_numpy(self):
        if self.fd_data is None:
            return None
        return namedtuple("DataContent", self.data_info.channels)(*self.fd_data.cpu().numpy())

    @property
    def fd_noise_power_density_numpy(self):
        if self.fd_noise_power_density is None:
            return None
        return namedtuple("DataContent", self.data_info.channels)(*self.fd_noise_power_density.cpu().numpy())


class TDICombinationModel(ABC):
    """tdi.py:1379-1385: the TDI plugin interface."""

    @abstractmethod
    def update_tdi_response(self):
        pass


class FDMichelsonConstantEqualArmFFT(TDICombinationModel):
    """tdi.py:1797-1810: a placeholder in the reference, as here (abstract:
    instantiating it raises TypeError, as there)."""


class FDMichelsonConstantEqualArm(TDICombinationModel):
    """tdi.py:1603-1793: FD Michelson TDI with constant equal arms."""

    domain = "fd"

    def __init__(self, generation="1.5", orthogonal=True, backend="cuda"):
        self.generation = str(generation)
        if self.generation not in ("1.5", "2.0"):
            raise ValueError(f"Unsupported generation {self.generation}.")
        if backend != "cuda":
            raise ValueError(f"Unknown backend: {backend}")
        self.orthogonal = bool(orthogonal)
        self.labels = ("A", "E", "T") if self.orthogonal else ("X", "Y", "Z")
        self.backend = backend
        self.detector = None

    @property
    def generation_code(self):
        return 15 if self.generation == "1.5" else 20

    def init_tdi_combination_model(self, detector):
        self.detector = detector
        n = detector.tdi_data.data_info.frequency_series_length
        detector.tdi_response = torch.zeros((3, n), dtype=torch.complex128, device="cuda")

    def update_tdi_response(self):
        det = self.detector
        freqs = det.tdi_data.frequency_samples
        n = freqs.numel()
        _lib.check(_lib.load().pes_tdi_combination(
            _lib.ptr(freqs), n, det.orbit_model.arm_length_sec(0.0), self.generation_code, int(self.orthogonal),
            _lib.ptr(det.single_link_response), _lib.ptr(det.tdi_response), _lib.stream_handle()))


class TDMichelsonConstantEqualArm(TDICombinationModel):
    """tdi.py:1388-1600: time-domain Michelson TDI with constant equal arms.

    The reference marks this class incomplete; the combination it defines is
    kept as written (``pes_td_tdi_combination``): output sample i combines the
    six single-link time series at sample i + ``added_time_samples_number``
    and, for k + 1 = 1..max_num_delay arm lengths, their linear interpolation
    between samples i + shift_k and i + shift_k + 1 with the reference's
    shifts and weights.  ``detector.single_link_response`` is a (6,
    ``extended_time_series_length``) float64 CUDA tensor in the order link12,
    link21, link23, link32, link31, link13; ``detector.tdi_response`` is the
    (3, ``time_series_length``) float64 result, rows in ``labels`` order.

    ``precision="fp64"`` (default) gives results bit-identical to the
    reference's operation order; ``"mixed"`` runs the combination in
    float-float arithmetic (``pes_td_tdi_combination_mixed``: within 2e-12 of
    the largest link magnitude it reads, several times faster on GB300, whose
    FP64 rate is 1/64 of FP32).
    """

    domain = "td"

    def __init__(self, generation="1.5", orthogonal=True, backend="cuda", precision="fp64"):
        self.generation = str(generation)
        if self.generation == "1.5":
            self.max_num_delay = 3
        elif self.generation == "2.0":
            self.max_num_delay = 7
        else:
            raise ValueError(f"Unsupported generation {self.generation}.")
        if backend != "cuda":
            raise ValueError(f"Unknown backend: {backend}")
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"Unknown precision: {precision}")
        self.orthogonal = bool(orthogonal)
        self.labels = ("A", "E", "T") if self.orthogonal else ("X", "Y", "Z")
        self.backend = backend
        self.precision = precision
        self.detector = None
        self.added_time_samples_number = None
        self.extended_time_series_length = None

    @property
    def generation_code(self):
        return 15 if self.generation == "1.5" else 20

    @staticmethod
    def _arm_sec(orbit_model):
        arm = getattr(orbit_model, "armlength_sec", None)
        if arm is None:
            arm = orbit_model.arm_length_sec(0.0)
        return float(arm)

    def init_tdi_combination_model(self, detector):
        self.detector = detector
        info = detector.tdi_data.data_info
        n = int(info.time_series_length)
        self.added_time_samples_number = int(
            self.max_num_delay * self._arm_sec(detector.orbit_model) // info.delta_time + 1)
        self.extended_time_series_length = int(n + self.added_time_samples_number)
        detector.tdi_response = torch.zeros((3, n), dtype=torch.float64, device="cuda")

    def update_tdi_response(self):
        det = self.detector
        links = det.single_link_response
        out = det.tdi_response
        n, n_ext = out.shape[-1], links.shape[-1]
        if links.dtype != torch.float64 or not links.is_cuda or links.shape[-2:] != (6, n_ext) \
                or not links.is_contiguous():
            raise ValueError("single_link_response must be a contiguous (6, n_ext) float64 CUDA tensor")
        lib = _lib.load()
        fn = lib.pes_td_tdi_combination if self.precision == "fp64" else lib.pes_td_tdi_combination_mixed
        _lib.check(fn(_lib.ptr(links), 1, n_ext, n, self._arm_sec(det.orbit_model),
                      float(det.tdi_data.data_info.delta_time), self.generation_code, int(self.orthogonal),
                      _lib.ptr(out), _lib.stream_handle()))
