"""CUDA plugin entry points against the oracle and the reference golden vectors.

Bar: orbits and grids bit-for-bit up to libm differences (<= 4e-15 relative),
links/TDI 1e-13 of the per-bin link scale, PhenomD container 1e-10 relative,
Whittle lnL 1e-12 relative.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from pespace_gb300 import _lib  # noqa: E402


def cuda(a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def orbit_c(kind_args):
    from pespace_gb300.detector.orbit import KaplerianHeliocentric, KeplerianGeocentric

    kind, args = kind_args
    return (KaplerianHeliocentric if kind == "helio" else KeplerianGeocentric)(*args)


ORBITS = {
    "lisa": ("helio", (2.5e9, 0.0, -np.pi / 9)),
    "taiji": ("helio", (3.0e9, 0.0, np.pi / 9)),
    "tianqin": ("geo", (np.sqrt(3.0) * 1e8, 0.3, 0.2)),
    "helio_rot": ("helio", (2.5e9, 0.7, 1.1)),
}


def test_orbit_vectors(cuda_lib, golden):
    for name, ka in ORBITS.items():
        orb = orbit_c(ka)
        v = orb.get_constellation_vectors(golden["orbit_times"])
        got = torch.stack(list(v), dim=1).cpu().numpy()
        ref = golden[f"orbit_{name}"]
        np.testing.assert_allclose(got, ref, rtol=4e-15, atol=4e-15 * np.abs(ref).max())


def test_polarization_host(cuda_lib, golden):
    from pespace_gb300.detector.antenna import get_gw_propagation_unit_vector, get_polarization_tensor_ssb

    for i, (lam, beta, psi) in enumerate(golden["pol_angles"]):
        P, X = get_polarization_tensor_ssb(lam, beta, psi)
        np.testing.assert_allclose(P, golden["pol_plus"][i], rtol=0, atol=4e-16)
        np.testing.assert_allclose(X, golden["pol_cross"][i], rtol=0, atol=4e-16)
        np.testing.assert_allclose(get_gw_propagation_unit_vector(lam, beta), golden["prop_k"][i], atol=4e-16)


@pytest.mark.parametrize("det", ["lisa", "tianqin"])
@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [1, 0])
def test_response_and_tdi_vs_golden(cuda_lib, golden, oracle, det, gen, orth):
    lib = _lib.load()
    orb = orbit_c(ORBITS[det])
    fr = cuda(golden["resp_freqs"])
    n = fr.numel()
    hp = cuda(golden["resp_wf_plus"][None], torch.complex128)
    hc = cuda(golden["resp_wf_cross"][None], torch.complex128)
    tf = cuda(golden["resp_wf_tf"][None], torch.float64)
    lam, beta, psi, tc = golden["resp_extrinsic"]
    links = torch.empty((6, n), dtype=torch.complex128, device="cuda")
    _lib.check(lib.pes_response_links(orb.to_c(), _lib.ptr(fr), n, 1, _lib.ptr(hp), _lib.ptr(hc), _lib.ptr(tf),
                                      lam, beta, psi, tc, _lib.ptr(links), None))
    out = torch.empty((3, n), dtype=torch.complex128, device="cuda")
    _lib.check(lib.pes_tdi_combination(_lib.ptr(fr), n, orb.orbit_params.static_arm_sec, 15 if gen == "1.5" else 20,
                                       orth, _lib.ptr(links), _lib.ptr(out), None))
    torch.cuda.synchronize()
    key = f"resp_{det}_{gen}_{orth}"
    ref_l = golden[key + "_links"]
    scale = np.sum(np.abs(ref_l), axis=0) + 1e-300
    L = links.cpu().numpy()
    assert np.max(np.abs(L - ref_l) / scale) < 1e-13
    T = out.cpu().numpy()
    assert np.max(np.abs(T - golden[key + "_tdi"]) / (4 * scale)) < 1e-13
    # and against the oracle on the same inputs
    oL = oracle.response_links(getattr(oracle, "heliocentric" if ORBITS[det][0] == "helio" else "geocentric")(
        *ORBITS[det][1]), golden["resp_freqs"], golden["resp_wf_plus"], golden["resp_wf_cross"],
        golden["resp_wf_tf"], lam, beta, psi, tc)
    assert np.max(np.abs(L - oL) / scale) < 1e-13


def test_multimode_and_empty(cuda_lib, golden):
    lib = _lib.load()
    orb = orbit_c(ORBITS["lisa"])
    fr = cuda(golden["resp_freqs"])
    n = fr.numel()
    hp = cuda(golden["mm_wf_plus"], torch.complex128)
    hc = cuda(golden["mm_wf_cross"], torch.complex128)
    tf = cuda(golden["mm_wf_tf"], torch.float64)
    lam, beta, psi, tc = golden["mm_extrinsic"]
    links = torch.empty((6, n), dtype=torch.complex128, device="cuda")
    _lib.check(lib.pes_response_links(orb.to_c(), _lib.ptr(fr), n, 2, _lib.ptr(hp), _lib.ptr(hc), _lib.ptr(tf),
                                      lam, beta, psi, tc, _lib.ptr(links), None))
    torch.cuda.synchronize()
    scale = np.sum(np.abs(golden["mm_links"]), axis=0) + 1e-300
    assert np.max(np.abs(links.cpu().numpy() - golden["mm_links"]) / scale) < 1e-13
    # empty inputs are a no-op; bad mode count is rejected
    assert lib.pes_response_links(orb.to_c(), None, 0, 1, None, None, None, 0.0, 0.0, 0.0, 0.0, None, None) == 0
    assert lib.pes_response_links(orb.to_c(), _lib.ptr(fr), n, 0, _lib.ptr(hp), _lib.ptr(hc), _lib.ptr(tf),
                                  0.0, 0.0, 0.0, 0.0, _lib.ptr(links), None) == _lib.PES_EINVAL


def test_whittle_kernel(cuda_lib, golden, oracle):
    from pespace_gb300.inference import noise_weighted_inner_product

    v = noise_weighted_inner_product(golden["nwip_d"], golden["nwip_h"], golden["nwip_s"], 0.125)
    assert abs(v - float(golden["nwip_value"])) <= 1e-12 * abs(v)
    # large ragged case vs oracle; deterministic across calls
    rng = np.random.default_rng(7)
    n = 300_001
    d = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    h = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    s = rng.uniform(0.1, 3.0, size=(3, n))
    a = noise_weighted_inner_product(d, h, s, 1e-3)
    b = noise_weighted_inner_product(d, h, s, 1e-3)
    assert a == b
    assert abs(a - oracle.whittle(d, h, s, 1e-3)) <= 1e-12 * abs(a)
    for C in (1, 2):
        v = noise_weighted_inner_product(d[:C], h[:C], s[:C], 1e-3)
        assert abs(v - oracle.whittle(d[:C], h[:C], s[:C], 1e-3)) <= 1e-12 * abs(v)
    assert noise_weighted_inner_product(d[:, :0], h[:, :0], s[:, :0], 1e-3) == 0.0


@pytest.mark.parametrize("q,c1,c2", [(2.0, 0.5, -0.3), (1.0, 0.0, 0.0), (7.5, 0.95, -0.9), (1.3, -0.98, 0.97)])
def test_phenomd_container(cuda_lib, oracle, q, c1, c2):
    from pespace_gb300.waveform import IMRPhenomD
    from tests.helpers import config0_theta

    th = config0_theta(3.0e6)
    th[1], th[2], th[3] = q, c1, c2
    g = oracle.grid(2.0 ** 22, 8.0, 1e-4, 0.03)
    wf = IMRPhenomD(g["freqs"], 1e-4)
    out = wf.from_theta(th)
    torch.cuda.synchronize()
    hp, hc, tf, _ = oracle.phenomd(th, g["freqs"], 1e-4)
    gp = out["plus"].cpu().numpy()
    gc = out["cross"].cpu().numpy()
    gt = out["tf"].cpu().numpy()
    amp = np.abs(hp)
    live = amp > 0
    assert np.array_equal(np.abs(gp) > 0, live)
    assert np.max(np.abs(gp - hp)[live] / amp[live]) < 1e-10
    assert np.max(np.abs(gc - hc)[live] / (np.abs(hc)[live] + 1e-300)) < 1e-10
    np.testing.assert_allclose(gt, tf, rtol=1e-10, atol=1e-9)
