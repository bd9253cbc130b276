"""Time-domain side of the data container (TDIChannelData, tdi.py:330-414,
521-583, 661-770): rfft of the windowed series over the sampling frequency,
cropped to the frequency mask; the unimplemented conversions raise as in the
reference.  CPU: the transform and the argument checks; GPU: the container
round trip."""

import numpy as np
import pytest

from pespace_gb300.detector.tdi import DataInformation, TDIChannelData, fd_from_td

T, DT = 4096.0, 2.0


def _info(fmin=1e-3, fmax=0.2):
    return DataInformation(("A", "E", "T"), T, DT, 0.0, fmin, fmax)


@pytest.mark.parametrize("window", [None, "hann", ("tukey", 0.1)])
def test_transform_matches_numpy(window):
    from scipy import signal

    info = _info()
    x = np.random.default_rng(3).standard_normal((3, info.time_series_length))
    w = np.ones(info.time_series_length) if window is None else signal.get_window(window, info.time_series_length)
    want = np.stack([(np.fft.rfft(r * w) / info.sampling_frequency)[info.frequency_mask_array] for r in x])
    got = fd_from_td(x, info, window)
    assert got.dtype == np.complex128 and got.shape == (3, info.frequency_series_length)
    assert np.array_equal(got, want)
    assert np.array_equal(fd_from_td(x, info, w), want)  # an explicit weight array


def test_cosine_at_a_bin_frequency():
    """x = cos(2 pi f_k t) at the k-th rfft frequency gives N / (2 f_s) at bin k."""
    info = _info(0.0, 1.0)
    n = info.time_series_length
    k = 37
    t = np.arange(n) * DT
    x = np.cos(2 * np.pi * (k / (n * DT)) * t)[None].repeat(3, axis=0)
    fd = fd_from_td(x, info)
    assert np.argmax(np.abs(fd[0])) == k
    assert abs(fd[0, k] - n / 2 / info.sampling_frequency) < 1e-9 * n
    others = np.delete(np.abs(fd[0]), k)
    assert np.max(others) < 1e-9 * n


def test_container_checks_without_a_device():
    td = TDIChannelData()
    with pytest.raises(ValueError):
        td.set_fd_data_from_td()  # no td_data yet
    with pytest.raises(ValueError):
        td.set_td_data_from_input(("A", "E"), T, DT, np.zeros((3, int(T // DT + 1))))  # channel count
    td2 = TDIChannelData()
    with pytest.raises(ValueError):
        td2.set_td_data_from_input(("A", "E", "T"), T, DT, np.zeros((3, 10)))  # series length
    for name in ("set_td_data_from_fd", "set_wd_data_from_zero", "set_wd_data_from_td", "set_wd_data_from_fd",
                 "set_fd_noise_power_density_from_td_data", "get_td_noise_realization"):
        with pytest.raises(NotImplementedError):
            getattr(TDIChannelData(), name)()
    assert TDIChannelData().td_data_numpy is None


@pytest.mark.gpu
def test_container_round_trip(cuda_lib):
    info = _info()
    x = np.random.default_rng(8).standard_normal((3, info.time_series_length))
    td = TDIChannelData()
    td.set_td_data_from_input(("A", "E", "T"), T, DT, x, 0.0, 1e-3, 0.2)
    assert td.td_data.is_cuda and np.array_equal(td.td_data_numpy.A, x[0])
    td.set_fd_data_from_td("hann")
    assert td.fd_data.is_cuda and np.array_equal(td.fd_data.cpu().numpy(), fd_from_td(x, info, "hann"))
    assert np.array_equal(td.frequency_samples.cpu().numpy(), info.frequency_samples_array)
    with pytest.raises(ValueError):
        td.set_fd_data_from_td()  # fd_data already set
    z = TDIChannelData()
    z.set_td_data_from_zero(("A", "E", "T"), T, DT)
    assert z.td_data.shape == (3, info.time_series_length) and not z.td_data.any()
