"""Roofline bookkeeping for bench.py: algorithmic work per kernel launch.

Mixed plan, kernel class ``dense_mixed`` (one ``k_dense_mixed`` launch per
call).  Its bins are compute work on data that stays in L2 (125410 bins x
48 B per detector, three float4 rows per bin), so the bound is the FP32 pipe.  FP32 arithmetic per bin
and detector, counted from the kernel source (FMA = 2 flops, add/mul = 1):

  phase advance from the run's anchor, error-free: three exact
    2 pi reductions of the split products (16 each), the products
    and powers of the lane index 5, a two-sum chain 18, the tails'
    polynomial 6 and their sum 5                                      82
  FMA-only sincos of the advance 29, first-order tail correction 4   33
  rotation by the run's anchor phasor 6, renormalisation 9, TDI
    generation prefactor 6                                           21
  kink coordinate 3, midpoint correction (bump shape 4, six
    products 6)                                                      13
  per channel (x3): spline value with the kink and midpoint terms
    24, model rotation 6, residual 2, |d - h|^2 w 5, |h|^2 w, the
    cross term and Re(d* h) w 14                            51 x 3 = 153
  weak-template branch 8, compensated sums (direct 4, cross 5)      17
  rounding estimate sum |d|^2 |h|^2 w^2 (7 x 3 + 1), which chooses
    the samples re-evaluated after the dense stage                   22
                                                       lnL pass:    341
  gradient pass: per-channel adjoints 13 x 3 = 39, interval moments
    (7 quantities x t^0..t^3) 58                              +97 = 438

The per-bin kink moments of post-peak bins are not counted (a lower bound).
The FP64 run anchors (about 30 FP64 operations per run of <= 32 bins) are
not in the FP32 count either.

Peak: cuBLAS SGEMM 8192^3 with TF32 off, measured in bench.py (FP32 pipe).
Traffic: DRAM bytes per dense bin measured by ncu on a 256-sample batch of
the same workload (dram__bytes_read.sum + dram__bytes_write.sum of one
k_dense_mixed<1> launch divided by its 19 603 667 dense bins); scaled here by
the launch's dense bins.
"""

FP32_FLOPS_PER_DENSE_BIN = {"lnl": 341, "grad": 438}
DRAM_BYTES_PER_DENSE_BIN = 5.69  # (103.32 MB + 8.18 MB) / 19 603 667 bins, ncu, 256 samples


def roofline(kernel_class, launches_ms, steps, work, grad, fp32_peak_tflops):
    """Roofline entry for the dominant kernel.

    kernel_class: profiler class name; launches_ms: (launches, summed device ms)
    over the timed steps; steps: timed steps; work: WhittleLikelihood.last_work()
    of one step; grad: whether the step ran the gradient pass.  A step may run
    the kernel more than once (a large batch runs as two halves), so the
    achieved rate is the step's work over the step's summed kernel time, and
    the work and traffic are given per launch.
    """
    launches, ms = launches_ms
    per_launch_ms = ms / max(1, launches)
    per_step_ms = ms / max(1, steps)
    per_step_launches = launches / max(1, steps)
    entry = {"kernel": kernel_class, "launches": launches, "avg_launch_ms": per_launch_ms,
             "bound": None, "unit": "TFLOP/s", "peak": None, "peak_source": None, "achieved": None,
             "frac": None, "traffic": None, "units_per_launch": None}
    if kernel_class == "dense_mixed":
        bins = work["dense_bins"] / per_step_launches
        flops = bins * FP32_FLOPS_PER_DENSE_BIN["grad" if grad else "lnl"]
        entry.update(bound="fp32", peak=fp32_peak_tflops,
                     peak_source="measured cuBLAS SGEMM 8192^3 (TF32 off) in bench.py",
                     units_per_launch={"dense_bins": bins, "fp32_flops": flops})
        entry["achieved"] = flops * per_step_launches / (per_step_ms / 1e3) / 1e12
        if fp32_peak_tflops:
            entry["frac"] = entry["achieved"] / fp32_peak_tflops
        if DRAM_BYTES_PER_DENSE_BIN is not None:
            entry["traffic"] = DRAM_BYTES_PER_DENSE_BIN * bins
    return entry


# Time-domain TDI (k_td_tdi): FP64 operations per output sample, counted from
# the kernel source.  For max_delay m: 6 differences of neighbouring link
# samples (staged once per sample and shared by the delays), 6 m
# interpolations of 2 operations (multiply, add), 3 channels of 2 (m + 1) - 1
# signed sums, and the A/E/T combination (7 adds/multiplies and 3 divisions,
# one operation each).  The operation order is the reference's, kept for
# bit-identical results, so none of them contract into FMAs.
def td_tdi_fp64_ops_per_sample(max_delay):
    return 6 + 2 * 6 * max_delay + 3 * (2 * (max_delay + 1) - 1) + 10


# DRAM bytes of one k_td_tdi<7> launch over 8 388 609 output samples (ncu
# --set full: 402.73 MB read + 167.52 MB written), per output sample.  The
# algorithmic figure is 72 B (six 8-byte link samples read, three written);
# part of the last writes is still in L2 when the kernel ends.
TD_TDI_DRAM_BYTES_PER_SAMPLE = (402.726144e6 + 167.52e6) / 8388609
