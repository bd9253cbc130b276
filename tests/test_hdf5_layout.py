"""HDF5 save/recover of the data container (tdi.py:1022-1292).

h5py is not installed here, so the tests drive the writer and reader through
an in-memory stand-in of the h5py calls they use: File(name, "x" | "r") as
a context manager, create_dataset with "a/b/c" paths, path lookup, group
membership, and dataset[()], which returns bytes for variable-length strings
as h5py 3 does.  They check the reference's layout (group and dataset names,
data_info fields in its order), the round trip, and the reference's recovery
checks.
"""

import sys
import types

import numpy as np
import pytest

from pespace_gb300.detector import tdi

REFERENCE_INFO_FIELDS = ("channels", "duration", "delta_time", "start_time", "minimum_frequency",
                         "maximum_frequency", "sampling_frequency", "delta_frequency", "time_series_length",
                         "time_samples_array", "full_frequency_series_length", "full_frequency_samples_array",
                         "frequency_mask_array", "frequency_samples_array", "frequency_series_length")


class _Dataset:
    def __init__(self, data):
        self.data = np.array(data, copy=True)

    def __getitem__(self, key):
        assert key == ()
        d = self.data
        if d.dtype == object:  # variable-length strings read back as bytes
            enc = np.vectorize(lambda x: x.encode("utf-8") if isinstance(x, str) else x, otypes=[object])
            d = enc(d)
        return d[()]


class _Group(dict):
    def _walk(self, path, create):
        node, parts = self, path.strip("/").split("/")
        for p in parts[:-1]:
            if not dict.__contains__(node, p):
                if not create:
                    raise KeyError(path)
                dict.__setitem__(node, p, _Group())
            node = dict.__getitem__(node, p)
        return node, parts[-1]

    def create_dataset(self, path, data):
        node, leaf = self._walk(path, True)
        if dict.__contains__(node, leaf):
            raise ValueError(f"{path} exists")
        dict.__setitem__(node, leaf, _Dataset(data))

    def __getitem__(self, path):
        node, leaf = self._walk(path, False)
        return dict.__getitem__(node, leaf)


class _Files:
    def __init__(self):
        self.store = {}

    def module(self):
        files = self

        class File(_Group):
            def __init__(self, name, mode):
                super().__init__()
                if mode == "x":
                    if name in files.store:
                        raise FileExistsError(name)
                    files.store[name] = self
                elif mode == "r":
                    self.update(files.store[name])
                else:
                    raise ValueError(mode)

            def __enter__(self):
                return self

            def __exit__(self, *exc):
                return False

        return types.SimpleNamespace(File=File, string_dtype=lambda encoding: object)


@pytest.fixture
def files(monkeypatch):
    f = _Files()
    monkeypatch.setitem(sys.modules, "h5py", f.module())
    return f


def _content(seed=0):
    info = tdi.DataInformation(("A", "E", "T"), 4096.0, 2.0, 10.0, 1e-3, 0.2)
    rng = np.random.default_rng(seed)
    n, nt = info.frequency_series_length, info.time_series_length
    arrays = {"td_data": rng.standard_normal((3, nt)),
              "fd_data": rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n)),
              "fd_noise_power_density": rng.uniform(1.0, 2.0, (3, n))}
    return info, arrays


def test_layout_and_round_trip(files):
    info, arrays = _content()
    tdi._hdf5_write("data.h5", True, "cuda", info, arrays)
    f = files.store["data.h5"]
    assert set(f) == {"class_attrs", "data_info", "tdi_data", "noise_data"}
    assert set(f["class_attrs"]) == {"scaling", "backend", "_np_fp", "_np_cp"}
    assert tuple(f["data_info"]) == REFERENCE_INFO_FIELDS
    assert set(f["tdi_data"]) == {"td_data", "fd_data"} and set(f["tdi_data/fd_data"]) == {"A", "E", "T"}
    assert set(f["noise_data"]) == {"fd_noise_power_density"}
    scaling, got, back = tdi._hdf5_read("data.h5")
    assert scaling is True
    for k in ("channels", "duration", "delta_time", "start_time", "minimum_frequency", "maximum_frequency"):
        assert getattr(got, k) == getattr(info, k), k
    assert np.array_equal(got.frequency_samples_array, info.frequency_samples_array)
    for k, v in arrays.items():
        assert np.array_equal(back[k], v), k
    with pytest.raises(FileExistsError):
        tdi._hdf5_write("data.h5", True, "cuda", info, arrays)


def test_partial_content(files):
    info, arrays = _content(1)
    tdi._hdf5_write("fd_only.h5", False, "cuda", info, {"fd_data": arrays["fd_data"]})
    scaling, _, back = tdi._hdf5_read("fd_only.h5")
    assert scaling is False and set(back) == {"fd_data"}


def test_recovery_checks(files):
    info, arrays = _content(2)
    tdi._hdf5_write("a.h5", False, "taichi", info, arrays)  # written by another backend: recovered all the same
    tdi._hdf5_read("a.h5")
    files.store["a.h5"]["class_attrs"]["_np_fp"] = _Dataset(np.array("float32", dtype=object))
    with pytest.raises(AssertionError, match="numerical precision"):
        tdi._hdf5_read("a.h5")
    tdi._hdf5_write("b.h5", False, "cuda", info, arrays)
    files.store["b.h5"]["data_info"]["frequency_series_length"] = _Dataset(np.array(info.frequency_series_length + 1))
    with pytest.raises(AssertionError, match="frequency_series_length"):
        tdi._hdf5_read("b.h5")


def test_without_h5py_the_calls_say_so():
    if "h5py" in sys.modules or __import__("importlib").util.find_spec("h5py") is not None:
        pytest.skip("h5py is installed")
    with pytest.raises(ImportError, match="h5py"):
        tdi.TDIChannelData().save_to_file("x.h5")
    with pytest.raises(ImportError, match="h5py"):
        tdi.TDIChannelData.recover_from_file("x.h5")
