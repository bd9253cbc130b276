"""CPU oracle of the time-domain Michelson TDI combination (test infrastructure only).

Restates ``TDMichelsonConstantEqualArm`` (pespace/detector/tdi.py:1388-1600),
which the reference marks incomplete; its arithmetic is followed as written:

* ``added`` = int(max_num_delay * armlength // delta_time + 1) extra link
  samples precede the output series (tdi.py:1449-1454), max_num_delay = 3
  for generation "1.5" and 7 for "2.0" (tdi.py:1419-1424);
* for delay k = 0..max_num_delay-1 (num_delay = k + 1) the fraction
  t_frac[k] = 1 - (num_delay * armlength % delta_time) / delta_time
  (tdi.py:1469-1480) and the left sample i + (max_num_delay - num_delay) *
  armlength // delta_time (tdi.py:1484-1491); the delayed link is
  left + (right - left) * t_frac[k] (tdi.py:1496-1500, utils.py:83-100);
* the undelayed sample is i + added (tdi.py:1502);
* X, Y, Z are the signed sums of tdi.py:1506-1591, evaluated left to right,
  and A = (Z - X)/sqrt 2, E = (X - 2Y + Z)/sqrt 6, T = (X + Y + Z)/sqrt 3
  (tdi.py:1593-1600).

The shifts and fractions are the reference's expressions on Python floats,
so Python's own ``//`` and ``%`` compute them here.  numpy's elementwise
operations round each step, like the left-to-right scalar evaluation.

Only ``tests/`` and ``bench.py``'s CPU baseline use this module, as the
checker of the CUDA kernel.
"""

import math

import numpy as np

LINKS = ("link12", "link21", "link23", "link32", "link31", "link13")


def max_num_delay(generation):
    generation = str(generation)
    if generation == "1.5":
        return 3
    if generation == "2.0":
        return 7
    raise ValueError(f"Unsupported generation {generation}.")


def layout(armlength_sec, delta_time, generation):
    """(added, shifts, fracs) as the reference computes them (Python floats)."""
    m = max_num_delay(generation)
    added = int(m * armlength_sec // delta_time + 1)
    fracs = [1.0 - (nd * armlength_sec % delta_time) / delta_time for nd in range(1, m + 1)]
    shifts = [int((m - nd) * armlength_sec // delta_time) for nd in range(1, m + 1)]
    return added, shifts, fracs


def combine(links, n, armlength_sec, delta_time, generation="1.5", orthogonal=True):
    """TDI channels (3, n) from single-link series links (6, n_ext), n_ext >= n + added.

    The link rows are in the order of ``LINKS``.  Returns (A, E, T) when
    ``orthogonal`` else (X, Y, Z).
    """
    links = np.asarray(links, dtype=np.float64)
    m = max_num_delay(generation)
    added, shifts, fracs = layout(armlength_sec, delta_time, generation)
    if links.shape[-1] < n + added:
        raise ValueError(f"{links.shape[-1]} link samples for {n} outputs, need n + {added}")
    i = np.arange(n)
    L = dict(zip(LINKS, links))
    cur = {k: v[i + added] for k, v in L.items()}
    # d[name][k]: link `name` delayed by k + 1 arm lengths
    d = {k: [] for k in LINKS}
    for k in range(m):
        left_i = i + shifts[k]
        for name, v in L.items():
            left, right = v[left_i], v[left_i + 1]
            d[name].append(left + (right - left) * fracs[k])
    l12, l21, l23, l32, l31, l13 = (cur[k] for k in LINKS)
    d12, d21, d23, d32, d31, d13 = (d[k] for k in LINKS)
    if str(generation) == "1.5":
        X = l13 + d31[0] + d12[1] + d21[2] - l12 - d21[0] - d13[1] - d31[2]
        Y = l21 + d12[0] + d23[1] + d32[2] - l23 - d32[0] - d21[1] - d12[2]
        Z = l32 + d23[0] + d31[1] + d13[2] - l31 - d13[0] - d32[1] - d23[2]
    else:
        X = (l13 + d31[0] + d12[1] + d21[2] + d12[3] + d21[4] + d13[5] + d31[6]
             - l12 - d21[0] - d13[1] - d31[2] - d13[3] - d31[4] - d12[5] - d21[6])
        Y = (l21 + d12[0] + d23[1] + d32[2] + d23[3] + d32[4] + d21[5] + d12[6]
             - l23 - d32[0] - d21[1] - d12[2] - d21[3] - d12[4] - d23[5] - d32[6])
        Z = (l32 + d23[0] + d31[1] + d13[2] + d31[3] + d13[4] + d32[5] + d23[6]
             - l31 - d13[0] - d32[1] - d23[2] - d32[3] - d23[4] - d31[5] - d13[6])
    if orthogonal:
        return np.stack([(Z - X) / math.sqrt(2.0), (X - 2.0 * Y + Z) / math.sqrt(6.0), (X + Y + Z) / math.sqrt(3.0)])
    return np.stack([X, Y, Z])
