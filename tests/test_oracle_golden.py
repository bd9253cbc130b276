"""Pins the CPU oracle to the reference: every array in tests/golden/ was
computed by the reference package's own code (tests/golden/make_golden.py)."""

import numpy as np
import pytest


def orbits(oracle):
    return {
        "lisa": oracle.heliocentric(2.5e9, 0.0, -np.pi / 9),
        "taiji": oracle.heliocentric(3.0e9, 0.0, np.pi / 9),
        "tianqin": oracle.geocentric(np.sqrt(3.0) * 1e8, 0.3, 0.2),
        "helio_rot": oracle.heliocentric(2.5e9, 0.7, 1.1),
    }


def test_orbits_bit_exact(oracle, golden):
    for name, desc in orbits(oracle).items():
        got = oracle.orbit_vectors(desc, golden["orbit_times"])
        np.testing.assert_array_equal(got, golden[f"orbit_{name}"])
        assert desc.arm_sec == float(golden[f"orbit_{name}_arm"])


def test_polarization(oracle, golden):
    for i, (lam, beta, psi) in enumerate(golden["pol_angles"]):
        P, X, k = oracle.polarization(lam, beta, psi)
        np.testing.assert_allclose(P, golden["pol_plus"][i], rtol=0, atol=2e-16)
        np.testing.assert_allclose(X, golden["pol_cross"][i], rtol=0, atol=2e-16)
        np.testing.assert_allclose(k, golden["prop_k"][i], rtol=0, atol=2e-16)


def test_grids_exact(oracle, golden):
    for i, case in enumerate(golden["grid_cases"]):
        g = oracle.grid(*case)
        meta = golden[f"grid{i}_meta"]
        assert (g["time_series_length"], g["full_length"], g["nbins"]) == tuple(int(x) for x in meta[:3])
        assert g["df"] == meta[3]
        if g["nbins"]:
            assert g["k0"] == int(meta[4])
        idx = g["k0"] + np.arange(g["nbins"])
        fk = idx * g["f_step"]  # the index arithmetic the kernels use
        if f"grid{i}_freqs" in golden.files:
            np.testing.assert_array_equal(fk, golden[f"grid{i}_freqs"])
        else:
            np.testing.assert_array_equal(fk[:32], golden[f"grid{i}_freqs_head"])
            np.testing.assert_array_equal(fk[-32:], golden[f"grid{i}_freqs_tail"])
            np.testing.assert_array_equal(fk[::997], golden[f"grid{i}_freqs_stride997"])


@pytest.mark.parametrize("name", ["lisa", "taiji", "tianqin_gwspace", "tianqin_sqrt3"])
def test_psd_exact(oracle, golden, name):
    kw = {"lisa": oracle.PSD_PRESETS["LISA_SciRDv1"], "taiji": oracle.PSD_PRESETS["Taiji_TDC"],
          "tianqin_gwspace": oracle.PSD_PRESETS["Tianqin_GWSpace"],
          "tianqin_sqrt3": dict(oms_level=1e-24, acc_level=1e-30, arm_length_sec=np.sqrt(3) * 1e8 / oracle.C_SI,
                                tianqin=True)}[name]
    for gen in ("1.5", "2.0"):
        for sc in (0, 1):
            d = oracle.psd(golden["psd_freqs"], "XYZAET", bool(sc), gen, **kw)
            np.testing.assert_array_equal(np.stack([d[c] for c in "XYZAET"]), golden[f"psd_{name}_{gen}_{sc}"])


def test_noise_realization_exact(oracle, golden):
    g = oracle.grid(2.0 ** 15, 8.0, 1e-4, 0.03)
    S = golden["noise_psd_lisa_15"]
    n = oracle.noise_realization(g, dict(zip("AET", S)), "AET", 2026)
    np.testing.assert_array_equal(np.stack([n[c] for c in "AET"]), golden["noise_seed2026_lisa_15"])


def _link_scale(links):
    return np.sum(np.abs(links), axis=0)


@pytest.mark.parametrize("det", ["lisa", "tianqin"])
@pytest.mark.parametrize("gen", ["1.5", "2.0"])
@pytest.mark.parametrize("orth", [1, 0])
def test_response_and_tdi(oracle, golden, det, gen, orth):
    desc = orbits(oracle)[det]
    fr = golden["resp_freqs"]
    lam, beta, psi, tc = golden["resp_extrinsic"]
    key = f"resp_{det}_{gen}_{orth}"
    L = oracle.response_links(desc, fr, golden["resp_wf_plus"], golden["resp_wf_cross"], golden["resp_wf_tf"],
                              lam, beta, psi, tc)
    ref_l = golden[key + "_links"]
    scale = _link_scale(ref_l) + 1e-300
    assert np.max(np.abs(L - ref_l) / scale) < 1e-13
    T = oracle.tdi(fr, desc.arm_sec, gen, orth, L)
    ref_t = golden[key + "_tdi"]
    assert np.max(np.abs(T - ref_t) / (4 * scale)) < 1e-13


def test_multimode_response(oracle, golden):
    desc = orbits(oracle)["lisa"]
    lam, beta, psi, tc = golden["mm_extrinsic"]
    L = oracle.response_links(desc, golden["resp_freqs"], golden["mm_wf_plus"], golden["mm_wf_cross"],
                              golden["mm_wf_tf"], lam, beta, psi, tc)
    scale = _link_scale(golden["mm_links"]) + 1e-300
    assert np.max(np.abs(L - golden["mm_links"]) / scale) < 1e-13
    T = oracle.tdi(golden["resp_freqs"], desc.arm_sec, "2.0", True, L)
    assert np.max(np.abs(T - golden["mm_tdi"]) / (4 * scale)) < 1e-13


def test_whittle_kernel(oracle, golden):
    v = oracle.whittle(golden["nwip_d"], golden["nwip_h"], golden["nwip_s"], 0.125)
    assert abs(v - float(golden["nwip_value"])) <= 1e-12 * abs(v)


def test_likelihood_cases(oracle, golden):
    """Full reference path (WhittleLikelihoodJax) incl. channel subsets and a 2-detector network."""
    orbs = {"lisa": orbits(oracle)["lisa"], "tianqin": orbits(oracle)["tianqin"]}
    fr = golden["resp_freqs"]
    ext = golden["lik_extrinsic"]
    for gen_f, nch, c0, net, wi, val in golden["lik_cases"]:
        gen = "1.5" if gen_f == 1.5 else "2.0"
        chans = {3: "AET", 2: "AE", 1: "T"}[int(nch)]
        idx = ["AET".index(c) for c in chans]
        total = 0.0
        for dn in (("lisa", "tianqin") if net else ("lisa",)):
            L = oracle.response_links(orbs[dn], fr, golden["lik_wf_plus"][int(wi)], golden["lik_wf_cross"][int(wi)],
                                      golden["lik_wf_tf"][int(wi)], *ext[int(wi)])
            h = oracle.tdi(fr, orbs[dn].arm_sec, gen, True, L)
            total += oracle.whittle(golden[f"lik_{gen}_data_{dn}"][idx], h[idx], golden[f"lik_{gen}_psd_{dn}"][idx],
                                    1 / 2.0 ** 15)
        assert abs(total - val) <= 1e-12 * abs(val)
