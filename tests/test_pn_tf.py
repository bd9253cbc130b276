"""Post-Newtonian t(f) of the lalsimulation interface (interface_lalsim.py:297-482).

CPU: the oracle against the reference's own outputs (``golden/reference_pn_tf.npz``,
made by ``golden/make_pn_tf.py``) and the C entry point's argument checks.
GPU: ``pes_pn_tf`` / ``get_PN_d_phase`` against the oracle.
"""

import os

import numpy as np
import pytest

from oracle import pn

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden_pn():
    return np.load(os.path.join(HERE, "golden", "reference_pn_tf.npz"))


def _rows(g):
    for i in range(len(g["mass_1"])):
        yield i, {k: float(g[k][i]) for k in ("mass_1", "mass_2", "spin_1z", "spin_2z")}, g["freqs"][i]


def _close(got, want, rtol):
    """|got - want| <= rtol max|want| per row (t(f) crosses zero at the ISCO)."""
    scale = np.max(np.abs(want), axis=-1, keepdims=True)
    return np.all(np.abs(got - want) <= rtol * scale), np.max(np.abs(got - want) / scale)


def test_oracle_matches_reference(golden_pn):
    for i, p, f in _rows(golden_pn):
        want = golden_pn["tf"][i]
        got = pn.pn_tf(p["mass_1"], p["mass_2"], p["spin_1z"], p["spin_2z"], f)
        assert np.array_equal(got == 0.0, want == 0.0)  # zero above the ISCO, nowhere else
        ok, err = _close(got, want, 1e-12)
        assert ok, (i, err)


def test_oracle_isco_and_above():
    m1, m2 = 6e5, 4e5
    f_isco = pn.X_ISCO / ((m1 + m2) * pn.MTSUN_SI)
    t = pn.pn_tf(m1, m2, 0.3, -0.2, np.array([0.5 * f_isco, f_isco * (1 - 1e-12), f_isco, 2 * f_isco]))
    assert t[0] < 0.0
    assert abs(t[1]) < 1e-6 * abs(t[0])
    assert t[2] == 0.0 and t[3] == 0.0


def test_entry_point_argument_checks():
    # host-side checks only (no launch): negative sizes and null pointers are rejected
    from pespace_gb300 import _lib

    lib = _lib.load()
    assert lib.pes_pn_tf(None, -1, None, 4, None, None) != 0
    assert b"pes_pn_tf" in lib.pes_last_error()
    assert lib.pes_pn_tf(None, 70000, None, 4, None, None) != 0
    assert lib.pes_pn_tf(None, 0, None, 0, None, None) == 0  # empty: nothing to do


@pytest.mark.gpu
def test_gpu_matches_oracle_golden_inputs(cuda_lib, golden_pn):
    from pespace_gb300.waveform import get_PN_d_phase

    for i, p, f in _rows(golden_pn):
        got = get_PN_d_phase(p, f)
        want = pn.pn_tf(p["mass_1"], p["mass_2"], p["spin_1z"], p["spin_2z"], f)
        assert got.shape == f.shape
        assert np.array_equal(got == 0.0, want == 0.0)
        ok, err = _close(got, want, 1e-12)
        assert ok, (i, err)
        ok, err = _close(got, golden_pn["tf"][i], 1e-12)
        assert ok, (i, err)


@pytest.mark.gpu
def test_gpu_batched_call(cuda_lib):
    import torch

    from pespace_gb300.waveform import get_PN_d_phase

    rng = np.random.default_rng(7)
    B = 300
    mtot = 10.0 ** rng.uniform(4.5, 7.5, B)
    q = rng.uniform(1.0, 10.0, B)
    params = {"mass_1": mtot * q / (1 + q), "mass_2": mtot / (1 + q),
              "spin_1z": rng.uniform(-0.99, 0.99, B), "spin_2z": rng.uniform(-0.99, 0.99, B)}
    f = np.geomspace(2e-5, 0.5, 4099)
    got = get_PN_d_phase(params, f)
    want = pn.pn_tf(params["mass_1"], params["mass_2"], params["spin_1z"], params["spin_2z"], f)
    assert got.shape == (B, f.size)
    assert np.array_equal(got == 0.0, want == 0.0)
    ok, err = _close(got, want, 1e-12)
    assert ok, err
    # tensor in, CUDA tensor out; a single system gives a 1-D result
    t = get_PN_d_phase({k: v[3] for k, v in params.items()}, torch.as_tensor(f))
    assert isinstance(t, torch.Tensor) and t.is_cuda and t.shape == (f.size,)
    assert np.array_equal(t.cpu().numpy(), got[3])
    # empty frequency grid
    assert get_PN_d_phase({k: v[0] for k, v in params.items()}, np.zeros(0)).shape == (0,)
