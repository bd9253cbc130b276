"""Roofline bookkeeping for bench.py: algorithmic work per kernel launch.

The FP64 operation counts per unit of work are produced by counting the
operations of the templated physics code (see ``csrc/pes_census.cu``); until
that census exists for a kernel class, the roofline entry reports the
measured time and leaves the fraction empty.
"""

CENSUS = {}


def roofline(kernel_class, launches_ms, engine, theta, fp64_peak_tflops, peaks):
    launches, ms = launches_ms
    per_launch_ms = ms / max(1, launches)
    entry = {"kernel": kernel_class, "launches": launches, "avg_launch_ms": per_launch_ms,
             "bound": "fp64", "unit": "TFLOP/s", "peak": fp64_peak_tflops,
             "peak_source": "measured cuBLAS DGEMM 8192^3 in bench.py", "achieved": None, "frac": None,
             "traffic": None}
    c = CENSUS.get(kernel_class)
    if c is not None:
        flops = c(engine, theta)
        entry["achieved"] = flops / (per_launch_ms / 1e3) / 1e12
        entry["frac"] = entry["achieved"] / fp64_peak_tflops if fp64_peak_tflops else None
    return entry
