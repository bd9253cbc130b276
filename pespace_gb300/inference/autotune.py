"""Autotuner of a plan's launch options (``PES_OPT_*`` in pespace_gb300.h).

The options change speed only (bit-identical lnL; the gradient's FP32 moment
atomics may sum in another order):

* ``dense_stage`` (mixed plans): the gradient pass of the dense stage copies
  each run's inputs one run ahead into shared memory, or loads them
  directly.  Copying wins when the inputs stream from DRAM; direct loads win
  when they sit in L2.  The default is a size threshold (64 MB).
* ``sample_threads``: threads per block of the per-sample kernels (set-up,
  ranges, peak kink), whose FP64 chains run one per sample.

``autotune`` searches one option at a time (the others held at their current
values).  It times every candidate on the caller's batch with CUDA events on
the current stream: one warm-up call, then the median of ``reps`` calls.  It
keeps the fastest candidate in the plan.  Run it outside CUDA-graph capture;
a ``CapturedStep`` recorded afterwards uses the tuned launches.
"""

import ctypes

import numpy as np
import torch

from .. import _lib

OPTIONS = {"dense_stage": _lib.PES_OPT_DENSE_STAGE, "sample_threads": _lib.PES_OPT_SAMPLE_THREADS}
CANDIDATES = {"dense_stage": (0, 1), "sample_threads": (4, 8, 16, 32)}


def get_option(likelihood, name):
    """Current value of launch option ``name`` of a WhittleLikelihood's plan."""
    v = ctypes.c_int64()
    _lib.check(_lib.load().pes_plan_get_option(likelihood._plan, OPTIONS[name], ctypes.byref(v)))
    return int(v.value)


def set_option(likelihood, name, value):
    """Set launch option ``name`` of a WhittleLikelihood's plan."""
    _lib.check(_lib.load().pes_plan_set_option(likelihood._plan, OPTIONS[name], int(value)))


def _time(fn, theta, reps):
    fn(theta)
    ms = []
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn(theta)
        e.record()
        e.synchronize()
        ms.append(s.elapsed_time(e))
    return float(np.median(ms))


def autotune(likelihood, theta, grad=True, reps=5, candidates=None):
    """Tune ``likelihood``'s launch options on the (B, 11) batch ``theta``.

    grad : time the lnL+gradient call (True) or the lnL call.
    candidates : {name: values} to search (default ``CANDIDATES``);
        ``dense_stage`` is skipped for FP64 plans, which ignore it.

    Returns {name: {"chosen": value, "ms": {value: median ms per call}}}; the
    chosen values stay set in the plan.
    """
    if reps < 1:
        raise ValueError("reps must be >= 1")
    cands = dict(CANDIDATES if candidates is None else candidates)
    unknown = set(cands) - set(OPTIONS)
    if unknown:
        raise ValueError(f"unknown launch options: {sorted(unknown)}")
    if likelihood.precision != "mixed":
        cands.pop("dense_stage", None)
    theta = likelihood._prep(theta)[: likelihood.max_batch]
    fn = likelihood.log_likelihood_and_grad if grad else likelihood.log_likelihood_batch
    report = {}
    for name, values in cands.items():
        times = {}
        for v in values:
            set_option(likelihood, name, v)
            times[int(v)] = _time(fn, theta, reps)
        best = min(times, key=times.get)
        set_option(likelihood, name, best)
        report[name] = {"chosen": best, "ms": times}
    return report
