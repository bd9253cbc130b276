"""Time-domain Michelson TDI (TDMichelsonConstantEqualArm, tdi.py:1388-1600).

The reference marks the class incomplete and cannot run here (taichi is
absent), so no reference outputs pin it: the oracle restates its arithmetic
as written and is pinned by known answers.  With an arm length that is a whole
number of samples every interpolation weight is 1, and the combination is the
textbook TDI with delays of 1..max_num_delay arm lengths, checked here sample
by sample.  CPU: the oracle, the C layout helper against Python's own float
operators, the entry points' argument checks.  GPU: ``pes_td_tdi_combination``
bit-identical to the oracle (staged and L1 paths, both generations, both
channel sets, batched, full size); ``pes_td_tdi_combination_mixed``
(float-float) within 2e-12 of the largest link magnitude, with NaN inputs
reaching the same outputs as in the oracle.
"""

import ctypes
import math
import types

import numpy as np
import pytest

from oracle import td_tdi

LISA_ARM_SEC = 2.5e9 / 299792458.0


def _layout_c(lib, arm, dt, gen):
    added, maxd = ctypes.c_int64(), ctypes.c_int32()
    shifts, fracs = (ctypes.c_int64 * 7)(), (ctypes.c_double * 7)()
    rc = lib.pes_td_tdi_layout(arm, dt, 15 if gen == "1.5" else 20, ctypes.byref(added), ctypes.byref(maxd),
                               shifts, fracs)
    assert rc == 0, lib.pes_last_error()
    m = maxd.value
    return added.value, list(shifts[:m]), list(fracs[:m])


def test_layout_follows_python_float_semantics():
    from pespace_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(11)
    cases = [(1.0, 0.1), (0.3, 0.1), (8.0, 1.0), (8.0, 0.25), (LISA_ARM_SEC, 5.0), (LISA_ARM_SEC, 0.25),
             (10.0, 4.0), (0.5773502691896258, 0.1), (219.2, 1.0), (219.4, 1.0), (2.0, 3.0)]
    cases += [(float(a), float(d)) for a, d in zip(rng.uniform(0.1, 40.0, 200), rng.uniform(0.01, 10.0, 200))]
    cases += [(k * d, d) for k in (1, 3, 7, 9) for d in (0.1, 0.2, 0.3, 0.7, 1.1)]  # exact-multiple edges
    for arm, dt in cases:
        for gen in ("1.5", "2.0"):
            want = td_tdi.layout(arm, dt, gen)
            got = _layout_c(lib, arm, dt, gen)
            assert got[0] == want[0] and got[1] == want[1], (arm, dt, gen, got, want)
            assert np.array_equal(np.array(got[2]), np.array(want[2])), (arm, dt, gen)
            assert all(0 <= sh and sh + 1 <= got[0] for sh in got[1])  # reads stay in [i, i + added]
            assert all(0.0 < f <= 1.0 for f in got[2])
    # Python's // is not floor(a / b): 3.0 // 0.1 == 29.0 while 3.0 / 0.1 == 30.0
    assert td_tdi.layout(1.0, 0.1, "1.5")[0] == int(3 * 1.0 // 0.1 + 1) == 30


@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [True, False])
def test_oracle_constant_links_cancel(gen, orth):
    n = 50
    added = td_tdi.layout(LISA_ARM_SEC, 5.0, gen)[0]
    links = np.repeat(np.arange(1.0, 7.0)[:, None], n + added, axis=1)
    out = td_tdi.combine(links, n, LISA_ARM_SEC, 5.0, gen, orth)
    assert out.shape == (3, n) and np.all(out == 0.0)


@pytest.mark.parametrize("gen", ["1.5", "2.0"])
def test_oracle_whole_sample_arm_is_textbook_tdi(gen):
    # arm = 8 samples: every weight is 1, so delay k reads sample i + added - (k + 1) * 8
    dt, arm, n = 0.5, 4.0, 64
    q = round(arm / dt)
    added, shifts, fracs = td_tdi.layout(arm, dt, gen)
    assert all(f == 1.0 for f in fracs)
    rng = np.random.default_rng(3)
    links = rng.integers(-1000, 1000, size=(6, n + added)).astype(np.float64)
    y = dict(zip(td_tdi.LINKS, links))
    out = td_tdi.combine(links, n, arm, dt, gen, False)
    m = td_tdi.max_num_delay(gen)
    # X of the first-generation Michelson and its second-generation extension, delays in arm lengths
    x_plus = [("link13", 0), ("link31", 1), ("link12", 2), ("link21", 3)]
    x_minus = [("link12", 0), ("link21", 1), ("link13", 2), ("link31", 3)]
    if m == 7:
        x_plus += [("link12", 4), ("link21", 5), ("link13", 6), ("link31", 7)]
        x_minus += [("link13", 4), ("link31", 5), ("link12", 6), ("link21", 7)]
    relabel = {"1": "2", "2": "3", "3": "1"}

    def cyc(name, c):
        for _ in range(c):
            name = "link" + relabel[name[4]] + relabel[name[5]]
        return name

    for c in range(3):
        for i in range(n):
            t = i + added
            want = (sum(y[cyc(nm, c)][t - d * q] for nm, d in x_plus)
                    - sum(y[cyc(nm, c)][t - d * q] for nm, d in x_minus))
            assert out[c, i] == want, (c, i)


def _scalar_reference_loop(links, n, arm, dt, generation, orthogonal):
    """The loop body of tdi.py:1482-1600 for one sample at a time, on Python floats."""
    m = td_tdi.max_num_delay(generation)
    added = int(m * arm // dt + 1)
    t_frac = [1.0 - ((i + 1) * arm % dt) / dt for i in range(m)]
    y = dict(zip(td_tdi.LINKS, (list(map(float, row)) for row in links)))
    out = [[], [], []]
    for i in range(n):
        d = {name: [0.0] * m for name in td_tdi.LINKS}
        for num_delay in range(m, 0, -1):
            i_shift = int((m - num_delay) * arm // dt)
            for name in td_tdi.LINKS:
                left, right = y[name][i + i_shift], y[name][i + i_shift + 1]
                d[name][num_delay - 1] = left + (right - left) * t_frac[num_delay - 1]
        c = {name: y[name][i + added] for name in td_tdi.LINKS}
        d12, d21, d23, d32, d31, d13 = (d[k] for k in td_tdi.LINKS)
        X = c["link13"] + d31[0] + d12[1] + d21[2]
        Y = c["link21"] + d12[0] + d23[1] + d32[2]
        Z = c["link32"] + d23[0] + d31[1] + d13[2]
        if m == 7:
            X = X + d12[3] + d21[4] + d13[5] + d31[6]
            Y = Y + d23[3] + d32[4] + d21[5] + d12[6]
            Z = Z + d31[3] + d13[4] + d32[5] + d23[6]
        X = X - c["link12"] - d21[0] - d13[1] - d31[2]
        Y = Y - c["link23"] - d32[0] - d21[1] - d12[2]
        Z = Z - c["link31"] - d13[0] - d32[1] - d23[2]
        if m == 7:
            X = X - d13[3] - d31[4] - d12[5] - d21[6]
            Y = Y - d21[3] - d12[4] - d23[5] - d32[6]
            Z = Z - d32[3] - d23[4] - d31[5] - d13[6]
        if orthogonal:
            vals = ((Z - X) / math.sqrt(2.0), (X - 2.0 * Y + Z) / math.sqrt(6.0), (X + Y + Z) / math.sqrt(3.0))
        else:
            vals = (X, Y, Z)
        for k in range(3):
            out[k].append(vals[k])
    return np.array(out)


@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [True, False])
def test_oracle_equals_scalar_loop(gen, orth):
    arm, dt, n = LISA_ARM_SEC, 0.7, 40
    added = td_tdi.layout(arm, dt, gen)[0]
    links = np.random.default_rng(13).standard_normal((6, n + added)) * 1e-20
    assert np.array_equal(td_tdi.combine(links, n, arm, dt, gen, orth),
                          _scalar_reference_loop(links, n, arm, dt, gen, orth))


def test_oracle_rejects_short_series_and_generation():
    with pytest.raises(ValueError):
        td_tdi.combine(np.zeros((6, 10)), 10, LISA_ARM_SEC, 5.0, "1.5")
    with pytest.raises(ValueError):
        td_tdi.layout(1.0, 1.0, "3.0")


def test_entry_point_argument_checks():
    # host-side checks only: no launch happens for any of these calls
    from pespace_gb300 import _lib

    lib = _lib.load()
    added = td_tdi.layout(LISA_ARM_SEC, 5.0, "2.0")[0]
    f = lib.pes_td_tdi_combination
    assert f(None, 1, 100 + added, 100, LISA_ARM_SEC, 5.0, 30, 1, None, None) != 0  # generation
    assert b"generation" in lib.pes_last_error()
    assert f(None, 1, 100 + added, 100, LISA_ARM_SEC, 0.0, 20, 1, None, None) != 0  # dt
    assert f(None, 1, 100 + added, 100, float("nan"), 5.0, 20, 1, None, None) != 0  # arm
    assert f(None, 1, 99 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) != 0  # series too short
    assert b"need n +" in lib.pes_last_error()
    assert f(None, 70000, 100 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) != 0  # batch
    assert f(None, 1, 100 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) != 0  # null pointers
    assert f(None, 0, 100 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) == 0  # empty batch
    assert f(None, 1, added, 0, LISA_ARM_SEC, 5.0, 20, 1, None, None) == 0  # empty series
    huge = 512 * 0x7FFFFFFF + 1
    assert f(None, 1, huge + added, huge, LISA_ARM_SEC, 5.0, 20, 1, None, None) != 0  # beyond the grid
    assert b"launch grid" in lib.pes_last_error()


def test_mixed_entry_point_argument_checks():
    from pespace_gb300 import _lib

    lib = _lib.load()
    f = lib.pes_td_tdi_combination_mixed
    added = td_tdi.layout(LISA_ARM_SEC, 5.0, "2.0")[0]
    assert f(None, 1, 100 + added, 100, LISA_ARM_SEC, 5.0, 16, 1, None, None) != 0  # generation
    assert f(None, 1, 99 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) != 0  # series too short
    long_added = td_tdi.layout(219.4, 1.0, "2.0")[0]  # 1536: beyond the staged window
    assert f(None, 1, 100 + long_added, 100, 219.4, 1.0, 20, 1, None, None) != 0
    assert b"longest delay" in lib.pes_last_error()
    assert f(None, 0, 100 + added, 100, LISA_ARM_SEC, 5.0, 20, 1, None, None) == 0  # empty batch


def test_class_constructor():
    from pespace_gb300.detector.tdi import TDMichelsonConstantEqualArm

    m = TDMichelsonConstantEqualArm("2.0", False)
    assert m.domain == "td" and m.max_num_delay == 7 and m.labels == ("X", "Y", "Z")
    assert TDMichelsonConstantEqualArm().labels == ("A", "E", "T")
    with pytest.raises(ValueError):
        TDMichelsonConstantEqualArm("1.0")
    with pytest.raises(ValueError):
        TDMichelsonConstantEqualArm(backend="taichi")
    with pytest.raises(ValueError):
        TDMichelsonConstantEqualArm(precision="fp32")
    assert TDMichelsonConstantEqualArm(precision="mixed").precision == "mixed"


# ----------------------------------------------------------------------------- GPU


def _run_gpu(links, n, arm, dt, gen, orth, mixed=False):
    import torch

    from pespace_gb300 import _lib

    x = torch.as_tensor(links, device="cuda").contiguous()
    B = x.shape[0]
    out = torch.full((B, 3, n), float("nan"), dtype=torch.float64, device="cuda")
    lib = _lib.load()
    fn = lib.pes_td_tdi_combination_mixed if mixed else lib.pes_td_tdi_combination
    _lib.check(fn(_lib.ptr(x), B, x.shape[-1], n, arm, dt, 15 if gen == "1.5" else 20, int(orth), _lib.ptr(out),
                  _lib.stream_handle()))
    return out.cpu().numpy()


MIXED_TOL = 2e-12  # of the largest link magnitude: float-float, about 2^-46 per operation


@pytest.mark.gpu
@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [True, False])
@pytest.mark.parametrize("arm,dt,n", [
    (LISA_ARM_SEC, 5.0, 5000),          # LISA, fractional delays, ragged last tile
    (3e9 / 299792458.0, 0.25, 4096),    # Taiji, whole tiles
    (0.5773502691896258, 0.1, 1),       # TianQin, one sample
    (4.0, 0.5, 2049),                   # whole-sample delays
    (219.2, 1.0, 3000),                 # 2.0: window of 2048 samples, the largest staged
    (219.4, 1.0, 3000),                 # 2.0: 2049 samples, read through the L1
    (LISA_ARM_SEC, 0.002, 3000),        # long delays: L1 path for both generations
])
def test_gpu_matches_oracle(cuda_lib, gen, orth, arm, dt, n):
    added = td_tdi.layout(arm, dt, gen)[0]
    rng = np.random.default_rng(17)
    B = 3
    n_ext = n + added + 5  # longer series than needed are allowed
    links = rng.standard_normal((B, 6, n_ext)) * 1e-21
    got = _run_gpu(links, n, arm, dt, gen, orth)
    for b in range(B):
        want = td_tdi.combine(links[b], n, arm, dt, gen, orth)
        assert np.array_equal(got[b], want), (b, np.max(np.abs(got[b] - want)))


@pytest.mark.gpu
def test_gpu_full_size_series(cuda_lib):
    # T = 2^25 s at dt = 4 s (8 388 609 samples), LISA, second generation
    arm, dt, gen = LISA_ARM_SEC, 4.0, "2.0"
    n = int(2.0 ** 25 // dt + 1)
    added = td_tdi.layout(arm, dt, gen)[0]
    rng = np.random.default_rng(5)
    links = rng.standard_normal((1, 6, n + added))
    got = _run_gpu(links, n, arm, dt, gen, True)[0]
    step = 1 << 20
    for s in range(0, n, step):
        e = min(n, s + step)
        want = td_tdi.combine(links[0][:, s:e + added], e - s, arm, dt, gen, True)
        assert np.array_equal(got[:, s:e], want), s


@pytest.mark.gpu
def test_gpu_through_detector_class(cuda_lib):
    import torch

    from pespace_gb300.detector.orbit import KaplerianHeliocentric
    from pespace_gb300.detector.tdi import TDMichelsonConstantEqualArm

    dt, n = 5.0, 3001
    orbit = KaplerianHeliocentric(2.5e9, 0.0, -math.pi / 9)
    det = types.SimpleNamespace(
        tdi_data=types.SimpleNamespace(data_info=types.SimpleNamespace(time_series_length=n, delta_time=dt)),
        orbit_model=orbit)
    for gen in ("1.5", "2.0"):
        tdi = TDMichelsonConstantEqualArm(gen, True)
        tdi.init_tdi_combination_model(det)
        assert det.tdi_response.shape == (3, n)
        arm = orbit.arm_length_sec(0.0)
        assert tdi.added_time_samples_number == td_tdi.layout(arm, dt, gen)[0]
        rng = np.random.default_rng(9)
        links = rng.standard_normal((6, tdi.extended_time_series_length))
        det.single_link_response = torch.as_tensor(links, device="cuda")
        tdi.update_tdi_response()
        want = td_tdi.combine(links, n, arm, dt, gen, True)
        assert np.array_equal(det.tdi_response.cpu().numpy(), want)
    det.single_link_response = torch.zeros((6, 10), dtype=torch.float64, device="cuda")
    with pytest.raises(Exception):
        tdi.update_tdi_response()


@pytest.mark.gpu
@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [True, False])
@pytest.mark.parametrize("arm,dt,n", [
    (LISA_ARM_SEC, 5.0, 5000),
    (3e9 / 299792458.0, 0.25, 4096),
    (0.5773502691896258, 0.1, 1),
    (219.2, 1.0, 3000),                 # 2.0: the largest window
])
def test_gpu_mixed_within_tolerance(cuda_lib, gen, orth, arm, dt, n):
    added = td_tdi.layout(arm, dt, gen)[0]
    if 512 + added + 1 > 2048:
        pytest.skip("delay beyond the float-float kernel's window")
    rng = np.random.default_rng(19)
    B = 2
    links = rng.standard_normal((B, 6, n + added)) * 1e-21
    links[1] *= 10.0 ** rng.uniform(-12, 0, (6, n + added))  # wide dynamic range in the second series
    got = _run_gpu(links, n, arm, dt, gen, orth, mixed=True)
    for b in range(B):
        want = td_tdi.combine(links[b], n, arm, dt, gen, orth)
        err = np.max(np.abs(got[b] - want)) / np.max(np.abs(links[b]))
        assert err <= MIXED_TOL, (b, err)


@pytest.mark.gpu
def test_gpu_mixed_full_size_and_nan(cuda_lib):
    arm, dt, gen = LISA_ARM_SEC, 4.0, "2.0"
    n = int(2.0 ** 25 // dt + 1)
    added = td_tdi.layout(arm, dt, gen)[0]
    rng = np.random.default_rng(23)
    links = rng.standard_normal((1, 6, n + added)) * 3e-20
    links[0, 2, 777_777] = np.nan
    got = _run_gpu(links, n, arm, dt, gen, True, mixed=True)[0]
    scale = np.nanmax(np.abs(links))
    step = 1 << 20
    for s in range(0, n, step):
        e = min(n, s + step)
        want = td_tdi.combine(links[0][:, s:e + added], e - s, arm, dt, gen, True)
        assert np.array_equal(np.isnan(got[:, s:e]), np.isnan(want)), s
        ok = ~np.isnan(want)
        assert np.max(np.abs(got[:, s:e][ok] - want[ok])) <= MIXED_TOL * scale, s
    assert np.isnan(got).any()


@pytest.mark.gpu
def test_gpu_mixed_through_detector_class(cuda_lib):
    import torch

    from pespace_gb300.detector.orbit import KaplerianHeliocentric
    from pespace_gb300.detector.tdi import TDMichelsonConstantEqualArm

    dt, n = 5.0, 3001
    orbit = KaplerianHeliocentric(2.5e9, 0.0, -math.pi / 9)
    det = types.SimpleNamespace(
        tdi_data=types.SimpleNamespace(data_info=types.SimpleNamespace(time_series_length=n, delta_time=dt)),
        orbit_model=orbit)
    tdi = TDMichelsonConstantEqualArm("2.0", False, precision="mixed")
    tdi.init_tdi_combination_model(det)
    links = np.random.default_rng(29).standard_normal((6, tdi.extended_time_series_length))
    det.single_link_response = torch.as_tensor(links, device="cuda")
    tdi.update_tdi_response()
    want = td_tdi.combine(links, n, orbit.arm_length_sec(0.0), dt, "2.0", False)
    assert np.max(np.abs(det.tdi_response.cpu().numpy() - want)) <= MIXED_TOL * np.max(np.abs(links))
