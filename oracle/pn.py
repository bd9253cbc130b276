"""CPU oracle of the post-Newtonian time-frequency map t(f) (test infrastructure only).

Restates the reference's ``get_PN_d_phase``
(pespace/waveform/interface_lalsim.py:297-482): the aligned-spin TaylorF2
phase Psi(x) = sum_k (a_k + b_k ln(pi x)) x^((k-5)/3), x = M f (Buonanno,
Iyer, Ochsner, Pan & Sathyaprakash, PRD 80, 084043 (2009); spin terms as in
Blanchet, Living Rev. Relativ. 17, 2 (2014)), and

    t(f) = -M / (2 pi) [dPsi/dx (x) - dPsi/dx (x_ISCO)]  for x < x_ISCO = 6^-3/2 / pi,
    t(f) = 0                                               above,

so that t(f_ISCO) = 0.  The coefficient table has to match the reference's
term by term (it is the published TaylorF2 expansion the reference uses), so
its entries follow interface_lalsim.py:346-445; the evaluation is written
here as the derivative of the phase series.

Only ``tests/`` uses this module, as the checker of the CUDA kernel.
"""

import numpy as np

MTSUN_SI = 4.925490947641266978197229498498379006e-6  # pespace/utils/constants.py:37
EULER_GAMMA = 0.5772156649015329  # pespace/utils/constants.py:57
X_ISCO = 1.0 / (6.0 ** 1.5 * np.pi)


def taylorf2_coefficients(m1, m2, chi1, chi2):
    """(a_0..a_8, b_5, b_6, b_8) of Psi(x) = sum_k (a_k + b_k ln(pi x)) x^((k-5)/3)."""
    m1, m2, chi1, chi2 = (np.asarray(v, dtype=np.float64) for v in (m1, m2, chi1, chi2))
    mt = m1 + m2
    eta = m1 * m2 / (mt * mt)
    e2, e3 = eta * eta, eta * eta * eta
    dl = np.sqrt(1.0 - 4.0 * eta)
    xa, xs = 0.5 * (chi1 - chi2), 0.5 * (chi1 + chi2)
    pi = np.pi
    pfac = -3.0 / (128.0 * eta)
    # PN expansion coefficients (each times pi^((k-5)/3) below)
    c = {}
    c[0] = np.ones_like(eta)
    c[1] = np.zeros_like(eta)
    c[2] = 3715.0 / 756.0 + 55.0 / 9.0 * eta
    c[3] = -16.0 * pi + 113.0 / 3.0 * dl * xa + (113.0 / 3.0 - 76.0 / 3.0 * eta) * xs
    c[4] = (15293365.0 / 508032.0 + 27145.0 / 504.0 * eta + 3085.0 / 72.0 * e2
            + (-405.0 / 8.0 + 200.0 * eta) * xa * xa - 405.0 / 4.0 * dl * xa * xs
            + (-405.0 / 8.0 + 5.0 / 2.0 * eta) * xs * xs)
    b5 = ((38645.0 / 756.0 - 65.0 / 9.0 * eta) * pi
          + (-732985.0 / 2268.0 - 140.0 / 9.0 * eta) * dl * xa
          + (-732985.0 / 2268.0 + 24260.0 / 81.0 * eta + 340.0 / 9.0 * e2) * xs)
    c[6] = (11583231236531.0 / 4694215680.0 - 640.0 / 3.0 * pi * pi - 6848.0 / 21.0 * EULER_GAMMA
            + (-15737765635.0 / 3048192.0 + 2255.0 / 12.0 * pi * pi) * eta
            + 76055.0 / 1728.0 * e2 - 127825.0 / 1296.0 * e3 - np.log(2.0) * 13696.0 / 21.0
            + 2270.0 / 3.0 * pi * dl * xa + (2270.0 / 3.0 - 520.0 * eta) * pi * xs
            + (75515.0 / 144.0 - 8225.0 / 18.0 * eta) * dl * xs * xa
            + (75515.0 / 288.0 - 263245.0 / 252.0 * eta - 480.0 * e2) * xa * xa
            + (75515.0 / 288.0 - 232415.0 / 504.0 * eta + 1255.0 / 9.0 * e2) * xs * xs)
    b6 = -6848.0 / 63.0 * np.ones_like(eta)
    c[7] = ((77096675.0 / 254016.0 + 378515.0 / 1512.0 * eta - 74045.0 / 756.0 * e2) * pi
            + (-25150083775.0 / 3048192.0 + 26804935.0 / 6048.0 * eta - 1985.0 / 48.0 * e2) * dl * xa
            + (-25150083775.0 / 3048192.0 + 10566655595.0 / 762048.0 * eta - 1042165.0 / 3024.0 * e2
               + 5345.0 / 36.0 * e3) * xs
            - 1140.0 * pi * dl * xa * xs
            + (-570.0 + 2240.0 * eta) * pi * xa * xa + (-570.0 + 40.0 * eta) * pi * xs * xs
            + (14585.0 / 8.0 - 215.0 / 2.0 * eta) * dl * xa * xs * xs
            + (14585.0 / 8.0 - 7270.0 * eta + 80.0 * e2) * xa * xa * xs
            + (14585.0 / 24.0 - 2380.0 * eta) * dl * xa ** 3
            + (14585.0 / 24.0 - 475.0 / 6.0 * eta + 100.0 / 3.0 * e2) * xs ** 3)
    c[8] = ((233915.0 / 168.0 - 99185.0 / 252.0 * eta) * dl * xa
            + (233915.0 / 168.0 - 3970375.0 / 2268.0 * eta + 19655.0 / 189.0 * e2) * xs)
    a = np.zeros((9,) + eta.shape)
    for k in (0, 1, 2, 3, 4, 6, 7):
        a[k] = pfac * c[k] * pi ** ((k - 5) / 3.0)
    # the reference scales the 4PN spin-orbit term by pi^2 (interface_lalsim.py:435-444)
    a[8] = pfac * c[8] * pi * pi
    bl = {5: pfac * b5, 6: pfac * b6 * pi ** (1.0 / 3.0), 8: -a[8]}
    return a, bl


def dpsi_dx(a, bl, x):
    """d/dx of sum_k a_k x^((k-5)/3) + sum_k b_k ln(pi x) x^((k-5)/3) (k = 5, 6, 8)."""
    out = np.zeros(np.broadcast_shapes(np.shape(a[0]), np.shape(x)))
    for k in (0, 1, 2, 3, 4, 6, 7, 8):
        p = (k - 5) / 3.0
        out = out + p * a[k] * x ** (p - 1.0)
    lp = np.log(np.pi * x)
    out = out + bl[5] / x
    out = out + bl[6] * x ** (-2.0 / 3.0) * (lp / 3.0 + 1.0)
    out = out + bl[8] * (lp + 1.0)
    return out


def pn_tf(m1, m2, chi1, chi2, freqs):
    """t(f) [s] for each parameter set (leading axes) at freqs [Hz] (last axis)."""
    m1, m2, chi1, chi2 = (np.asarray(v, dtype=np.float64)[..., None] for v in (m1, m2, chi1, chi2))
    freqs = np.asarray(freqs, dtype=np.float64)
    msec = (m1 + m2) * MTSUN_SI
    x = freqs * msec
    a, bl = taylorf2_coefficients(m1, m2, chi1, chi2)
    d_isco = dpsi_dx(a, bl, np.full_like(x, X_ISCO))
    with np.errstate(divide="ignore", invalid="ignore"):
        d = dpsi_dx(a, bl, np.maximum(x, 1e-300))
    return np.where(x < X_ISCO, -msec / (2.0 * np.pi) * (d - d_isco), 0.0)
