"""Generate the golden fixture of the post-Newtonian t(f) map.

``reference_pn_tf.npz`` holds t(f) computed by the reference's own
``get_PN_d_phase`` (pespace/waveform/interface_lalsim.py:297-482), imported
from a checkout given on the command line with stand-ins for its absent
third-party modules (``_refshim.py``; lalsuite is replaced by empty modules,
which that function does not use).

Inputs are seeded: binary parameters over massive-black-hole and
stellar-mass ranges (detector-frame masses, aligned spins up to 0.99) and
frequency grids that cross each system's ISCO frequency.

Usage (needs the reference checkout; the fixture is committed):

    python tests/golden/make_pn_tf.py /path/to/pespace-checkout
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _refshim  # noqa: E402


def main(ref_root):
    _refshim.install(ref_root)
    sys.modules.setdefault("lal", types.ModuleType("lal"))
    sys.modules.setdefault("lalsimulation", types.ModuleType("lalsimulation"))
    from pespace.waveform.interface_lalsim import get_PN_d_phase

    rng = np.random.default_rng(2026)
    n_par = 24
    mtot = np.concatenate([10.0 ** rng.uniform(5.0, 7.0, 16), 10.0 ** rng.uniform(0.5, 2.0, 8)])
    q = rng.uniform(1.0, 8.0, n_par)
    m1 = mtot * q / (1.0 + q)
    m2 = mtot / (1.0 + q)
    chi1 = rng.uniform(-0.99, 0.99, n_par)
    chi2 = rng.uniform(-0.99, 0.99, n_par)
    chi1[0] = chi2[0] = 0.0
    m1[1] = m2[1] = 0.5 * mtot[1]  # equal masses (delta = 0)
    n_f = 257
    freqs = np.zeros((n_par, n_f))
    tf = np.zeros((n_par, n_f))
    for i in range(n_par):
        f_isco = 1.0 / (6.0 ** 1.5 * np.pi * mtot[i] * _refshim_mtsun())
        freqs[i] = np.geomspace(1e-3 * f_isco, 2.0 * f_isco, n_f)
        params = {"mass_1": m1[i], "mass_2": m2[i], "spin_1z": chi1[i], "spin_2z": chi2[i]}
        tf[i] = get_PN_d_phase(params, freqs[i])
    out = os.path.join(HERE, "reference_pn_tf.npz")
    np.savez_compressed(out, mass_1=m1, mass_2=m2, spin_1z=chi1, spin_2z=chi2, freqs=freqs, tf=tf)
    print("wrote", out, tf.shape)


def _refshim_mtsun():
    from pespace.utils.constants import MTSUN_SI

    return MTSUN_SI


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path to the pespace checkout>")
    main(sys.argv[1])
