/*
 * pespace_gb300 — C ABI of the GB300 (sm_103a) frequency-domain response and
 * Whittle-likelihood path of pespace.
 *
 * Conventions
 *  - Every function returns an int status: PES_OK (0) or one of the PES_E*
 *    codes below; none aborts the process.  pes_last_error() gives a message.
 *  - All array arguments are DEVICE pointers unless the comment says "host".
 *    The caller owns every input and output buffer.  Complex arrays are
 *    interleaved (re, im) doubles, i.e. the memory layout of complex128.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Launches are asynchronous on that stream; no function synchronises the
 *    device except pes_plan_create / pes_plan_set_data (set-up calls).
 *  - Channel-major layouts: a "(C, n)" array holds channel c at offset c*n.
 *
 * Source parameter vector ("theta", 11 doubles per sample, row-major (B, 11)):
 *   0 ln Mc [Msun, detector frame]   1 q = m1/m2 >= 1      2 chi1   3 chi2
 *   4 ln D_L [Mpc]                   5 cos(iota)           6 lambda (ecliptic longitude)
 *   7 sin(beta)                      8 psi                 9 phi_c  10 t_c [s]
 */
#ifndef PESPACE_GB300_H_
#define PESPACE_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PES_OK 0
#define PES_EINVAL 1   /* bad argument (sizes, pointers, enum values)           */
#define PES_ENOMEM 2   /* device allocation failed                              */
#define PES_ECUDA 3    /* a CUDA call failed                                    */
#define PES_ETIMEOUT 4 /* a bounded device wait gave up                         */

/* Per-sample status codes written by the batched calls. */
#define PES_SAMPLE_OK 0
#define PES_SAMPLE_NONFINITE 1
#define PES_SAMPLE_OUT_OF_DOMAIN 2

/* Analytic Keplerian constellation orbit.
 * kind 0: heliocentric (pespace/detector/orbit.py:155-241, KaplerianHeliocentric)
 * kind 1: geocentric   (pespace/detector/orbit.py:67-152,  KeplerianGeocentric)
 * Fields are the reference's `orbit_params` (orbit.py:112-140, 200-229). */
typedef struct PesOrbit {
  int32_t kind;
  int32_t pad;
  double arm_sec;             /* static_arm_sec = L / c                         */
  double rotation_initial;
  double revolution_initial;
  double omega_revolution;    /* 2 pi / year                                    */
  double r_sec;               /* heliocentric r' = L/(2 sqrt 3); geocentric L/sqrt 3 */
  double omega_rotation;      /* geocentric only                                */
  double slam_ref, clam_ref, sbeta_ref, cbeta_ref; /* geocentric reference frame */
  double ck[3], sk[3];        /* heliocentric node phases cos/sin(kappa_k)      */
} PesOrbit;

const char* pes_last_error(void);
int pes_version(void);

/* ---------------------------------------------------------------- plugins --
 * One call per reference plugin method; these are the drop-in entry points. */

/* Replaces the orbit model's get_constellation_vectors(time)
 * (pespace/detector/orbit.py:260-322, 362-419).  out: (n, 6, 3) doubles:
 * n1, n2, n3, x1, x2, x3 per time sample (light-seconds, SSB frame). */
int pes_orbit_vectors(const PesOrbit* orbit /* host */, const double* time, int64_t n, double* out,
                      void* stream);

/* Replaces get_polarization_tensor_ssb_taichi and
 * get_gw_propagation_unit_vector_taichi (pespace/detector/antenna.py:42-114).
 * All outputs host, row-major 3x3 and 3. */
int pes_polarization(double lam, double beta, double psi, double* plus9, double* cross9, double* k3);

/* Replaces FDResponseModelMarset2018.update_single_link_response(waveform, lam,
 * beta, psi, tc) (pespace/detector/antenna.py:403-543).  The waveform container
 * has n_modes modes: hp, hc (n_modes, n) complex; tf (n_modes, n) real.
 * links out: (6, n) complex in the order link12, 21, 23, 32, 31, 13. */
int pes_response_links(const PesOrbit* orbit /* host */, const double* freqs, int64_t n, int32_t n_modes,
                       const double* hp, const double* hc, const double* tf, double lam, double beta, double psi,
                       double tc, double* links, void* stream);

/* Replaces FDMichelsonConstantEqualArm.update_tdi_response()
 * (pespace/detector/tdi.py:1675-1793).  generation: 15 ("1.5") or 20 ("2.0").
 * orthogonal != 0 gives A, E, T; else X, Y, Z.  out: (3, n) complex. */
int pes_tdi_combination(const double* freqs, int64_t n, double arm_sec, int32_t generation, int32_t orthogonal,
                        const double* links, double* out, void* stream);

/* Replaces compute_whittle_likelihood_ti(channels, data, response, psd, df)
 * (pespace/inference/likelihood_ti.py:17-69): out[0] = -2 df sum |d-h|^2/S over
 * n_chan channels of (n_chan, n) arrays.  Deterministic two-pass sum; the
 * caller provides `workspace` of pes_whittle_workspace_len(n) doubles. */
int64_t pes_whittle_workspace_len(int64_t n);
int pes_whittle_lnl(const double* data, const double* response, const double* psd, int32_t n_chan, int64_t n,
                    double df, double* workspace, int64_t workspace_len, double* out, void* stream);

/* Allocation-free variant of pes_whittle_lnl (no counterpart in the reference).
 * For callers that may not allocate device memory at all: code running while a
 * stream is being captured into a CUDA graph (cudaMalloc is not permitted
 * there), and host runtimes that own the device memory pool and forbid
 * libraries from allocating (an XLA/JAX FFI custom call, a taichi-managed
 * context).  It needs no workspace argument: its scratch is a file-scope
 * device array of PES_WHITTLE_NOALLOC_PARTIALS doubles (8 KB) that every GPU
 * loading this library holds until the process exits.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress), so make
 * the first call on each device before any stream capture.  All calls share
 * the one array: calls whose kernels overlap on the GPU (different streams, or
 * host threads) race and must be serialised by the caller.  The scratch needs
 * no clearing (each call writes every partial it reads).
 * Limits: 1 <= n_chan <= 3, 0 <= n <= PES_WHITTLE_NOALLOC_MAX_BINS; sizes
 * outside them return PES_EINVAL with a message.  Calls no allocating routine. */
#define PES_WHITTLE_NOALLOC_PARTIALS 1024
#define PES_WHITTLE_NOALLOC_MAX_BINS 2147483647LL
int pes_whittle_lnl_noalloc(const double* data, const double* response, const double* psd, int32_t n_chan, int64_t n,
                            double df, double* out, void* stream);

/* Waveform producer (the external tiwave `update_waveform` contract used at
 * pespace/inference/interface_bilby.py:97; container layout antenna.py:438-458):
 * IMRPhenomD (2,2) plus/cross polarisations and t(f) at `freqs`, t_c = 0,
 * zero above f_cut_hz and above Mf = 0.2.  theta: host, 11 doubles. */
int pes_phenomd(const double* theta /* host */, const double* freqs, int64_t n, double f_ref, double f_cut_hz,
                double* hp, double* hc, double* tf, void* stream);

/* Higher-mode waveform producer: the mode-keyed container of the reference's
 * higher-mode producers (pespace/waveform/interface_ripple.py:155-235; consumed
 * mode by mode at antenna.py:446-458), with IMRPhenomHM (London et al. 2018)
 * in place of the absent IMRPhenomXHM.  Modes, in this order: (2,2), (2,1),
 * (3,3), (3,2), (4,4), (4,3).  hp, hc: (6, n) complex; tf: (6, n) seconds,
 * t_c = 0; each mode zero above f_cut_hz and above its mapped Mf = 0.2.
 * theta: host, 11 doubles. */
int pes_phenomhm(const double* theta /* host */, const double* freqs, int64_t n, double f_ref, double f_cut_hz,
                 double* hp, double* hc, double* tf, void* stream);

/* Post-Newtonian time-frequency map of the lalsimulation waveform interface:
 * replaces get_PN_d_phase (pespace/waveform/interface_lalsim.py:297-482),
 * which fills the `tf` entry of the waveform container for lalsimulation's FD
 * approximants (interface_lalsim.py:279-281).  params: device, (B, 4) doubles
 * (mass_1, mass_2 [Msun, detector frame], spin_1z, spin_2z); freqs: device,
 * (n) [Hz]; tf: device, (B, n) seconds, t(f_ISCO) = 0 and 0 above f_ISCO.
 * FP64.  1 <= B <= 65535 per call. */
int pes_pn_tf(const double* params, int64_t B, const double* freqs, int64_t n, double* tf, void* stream);

/* Time-domain Michelson TDI for constant equal arms: replaces
 * TDMichelsonConstantEqualArm.update_tdi_response() (pespace/detector/tdi.py:
 * 1460-1600; the reference marks the class incomplete, and its arithmetic is
 * followed as written).  links: device, (B, 6, n_ext) doubles, the single-link
 * time series in the order link12, 21, 23, 32, 31, 13 (utils.py:22-29);
 * out: device, (B, 3, n) doubles, A, E, T (orthogonal != 0) or X, Y, Z.
 * Output sample i reads link samples i .. i + added; n_ext >= n + added, where
 * added = int(max_delay * arm_sec // delta_time + 1) (tdi.py:1449-1454),
 * max_delay 3 (generation 15) or 7 (20).  FP64, bit-identical to the
 * reference's operation order.  0 <= B <= 65535. */
int pes_td_tdi_combination(const double* links, int64_t B, int64_t n_ext, int64_t n, double arm_sec,
                           double delta_time, int32_t generation, int32_t orthogonal, double* out, void* stream);

/* The same combination in float-float arithmetic on the FP32 pipe (no
 * counterpart in the reference; the FP64 entry point above is the drop-in).
 * Same arguments and layouts.  Each output is within about 2^-46 of the
 * magnitudes it combines: |out - exact| <= 2e-12 max |link| over the
 * samples it reads (the exact path is bit-identical).  Requires
 * added <= 1535 (e.g. sampling steps >= 0.04 s for LISA at generation 20). */
int pes_td_tdi_combination_mixed(const double* links, int64_t B, int64_t n_ext, int64_t n, double arm_sec,
                                 double delta_time, int32_t generation, int32_t orthogonal, double* out,
                                 void* stream);

/* Host only: the delay layout pes_td_tdi_combination uses, the reference's
 * expressions on Python floats (tdi.py:1449-1454, 1469-1491): added (above),
 * max_delay, and for delay k = 0 .. max_delay-1 the left sample offset
 * shifts[k] = (max_delay - k - 1) * arm_sec // delta_time and the weight
 * fracs[k] = 1 - ((k + 1) * arm_sec % delta_time) / delta_time of the right
 * sample.  shifts and fracs: host, 7 entries each. */
int pes_td_tdi_layout(double arm_sec, double delta_time, int32_t generation, int64_t* added, int32_t* max_delay,
                      int64_t* shifts, double* fracs);

/* ---------------------------------------------------------------- plans --
 * Batched lnL / lnL+gradient over B parameter samples: the per-sample loop of
 * LikelihoodBilbyInterfaceTaichi.log_likelihood (interface_bilby.py:78-116) and
 * WhittleLikelihoodJax.log_likelihood (likelihood_jax.py:207-260) fused into
 * one set of kernels per batch.  The plan owns its device workspaces. */

#define PES_MAX_DETECTORS 4
#define PES_PRECISION_FP64 0 /* dense FP64 evaluation on every bin             */
#define PES_PRECISION_MIXED 1 /* FP64 sparse grid + FP32 dense spline bulk      */
#define PES_APPROX_PHENOMD 0  /* IMRPhenomD, the (2,2) mode                       */
#define PES_APPROX_PHENOMHM 1 /* IMRPhenomHM, modes (2,2),(2,1),(3,3),(3,2),(4,4),(4,3) */

typedef struct PesDetectorDesc {
  PesOrbit orbit;
  int32_t generation; /* 15 or 20 */
  int32_t pad;
} PesDetectorDesc;

typedef struct PesPlanDesc {
  int64_t nbins;      /* dense bins in [fmin, fmax]                              */
  int64_t k0;         /* rfft index of the first bin                             */
  double f_step;      /* rfft spacing 1/(Nt dt): f_k = (k0 + i) f_step           */
  double df;          /* likelihood weight delta_frequency = 1/T (tdi.py:130)    */
  double f_ref;       /* waveform reference frequency [Hz]                       */
  double cut_factor;  /* per-sample model cutoff cut_factor * f_RD (0: Mf = 0.2) */
  int32_t n_det;
  int32_t chan_mask;  /* bit c: channel c of (A, E, T) enters lnL                */
  int32_t precision;  /* PES_PRECISION_*                                         */
  int32_t n_sparse;   /* mixed: sparse log-spaced nodes in [fmin, fmax]          */
  int32_t max_batch;  /* largest B passed to the batch calls                     */
  int32_t approximant; /* PES_APPROX_*: the waveform of the plan's samples         */
  PesDetectorDesc det[PES_MAX_DETECTORS];
} PesPlanDesc;

typedef struct PesPlan PesPlan;

int pes_plan_create(const PesPlanDesc* desc /* host */, PesPlan** plan /* host */);
int pes_plan_destroy(PesPlan* plan);
/* Copies detector `det`'s data (3, nbins) complex A/E/T and PSD (3, nbins) into
 * the plan (device pointers; synchronises `stream`). */
int pes_plan_set_data(PesPlan* plan, int32_t det, const double* data, const double* psd, void* stream);
/* lnl: (B,) ; status: (B,) int32 or NULL. */
int pes_lnl_batch(PesPlan* plan, const double* theta, int64_t B, double* lnl, int32_t* status, void* stream);
/* lnl and its gradient with respect to the 11 parameters; grad: (B, 11). */
int pes_lnl_grad_batch(PesPlan* plan, const double* theta, int64_t B, double* lnl, double* grad, int32_t* status,
                       void* stream);
/* Dense model of detector `det` for one parameter set (parity/debug path):
 * out (3, nbins) complex A/E/T (or X/Y/Z when orthogonal == 0). theta: host. */
int pes_plan_model_tdi(PesPlan* plan, int32_t det, int32_t orthogonal, const double* theta, double* out,
                       void* stream);

/* Measurement hooks (no counterpart in the reference).  While enabled, the plan
 * records a CUDA event pair on the caller's stream around every kernel it
 * launches.  pes_plan_stats (host; synchronises the recorded events) returns,
 * per kernel class k < PES_KERNEL_CLASSES, the launches and the summed device
 * milliseconds since the last reset, then resets them. */
#define PES_KERNEL_CLASSES 8
int pes_plan_profile(PesPlan* plan, int32_t enable);
int pes_plan_stats(PesPlan* plan, int64_t* launches /* host [8] */, double* device_ms /* host [8] */);
const char* pes_kernel_class_name(int32_t k);

/* Launch options of a plan (no counterpart in the reference).  They change
 * speed only: results agree bit for bit, except the gradient, whose FP32
 * moment atomics may sum in another order.  The Python autotuner
 * (pespace_gb300.inference.autotune) times the candidates on a caller's
 * batch and keeps the fastest.
 *   PES_OPT_DENSE_STAGE (mixed plans; FP64 plans read 0 and ignore it):
 *     1 = the gradient pass of the dense stage copies each run's inputs one
 *     run ahead into shared memory (cp.async), 0 = plain loads.  Default: 1
 *     when the packed dense inputs exceed 64 MB (they stream from DRAM).
 *   PES_OPT_SAMPLE_THREADS: threads per block of the per-sample kernels of
 *     the lnL calls (set-up, ranges, peak kink), 1..128 (the gradient
 *     set-up uses up to 255 registers per thread); default 8.
 * One option changes results, not speed, and is not tuned:
 *   PES_OPT_REFINE_ALL (mixed plans): 1 = every sample's dense range is
 *     re-evaluated as the samples whose error estimates approach the
 *     accuracy target always are: in float-float from its splines, or
 *     exactly where the splines' own error estimate exceeds the target (a
 *     check of those paths, and the most accurate mixed result at about
 *     twice the dense stage's cost); 0 (default) = only those samples. */
#define PES_OPT_DENSE_STAGE 1
#define PES_OPT_SAMPLE_THREADS 2
#define PES_OPT_REFINE_ALL 3
int pes_plan_set_option(PesPlan* plan, int32_t option, int64_t value);
int pes_plan_get_option(PesPlan* plan, int32_t option, int64_t* value /* host */);

/* Fisher matrices at B parameter sets (row-major (B, 11, 11), parameter order
 * of theta): F_ij = 4 df Re sum_{det, c, f} conj(dh_i) dh_j / S_c(f) over the
 * plan's channels and each sample's live bins.  FP64 plans take the
 * derivatives of the A/E/T model by FP64 forward-mode dual numbers; mixed
 * plans by the model's structure (PhenomD tangents in float-float, response
 * tangents in FP32; within a few 1e-6 of sqrt(F_ii F_jj) of the FP64 result).  The data are
 * not used, only the PSDs.  Replaces pespace/inference/fisher.py:27-162
 * (fisher_matrix).  Out-of-domain samples get NaN and their status.  The first
 * call allocates the plan's Fisher workspace (about 6 KB + 25 KB per sample of
 * max_batch). */
int pes_fisher_batch(PesPlan* plan, const double* theta, int64_t B, double* fisher /* (B,11,11) */,
                     int32_t* status /* nullable */, void* stream);

/* Work units of the last pes_lnl_batch / pes_lnl_grad_batch call of B samples
 * (host; synchronises `stream`), for roofline bookkeeping.  No reference
 * counterpart.  out[0]: bins through the mixed plan's FP32 dense stage,
 * summed over samples and detectors; out[1]: bins evaluated directly in FP64
 * (all live bins of an fp64 plan, the exact low-frequency bins of a mixed
 * plan); out[2]: sparse-node evaluations (mixed plans); out[3]: samples in
 * the parameter domain; out[4], out[5]: samples whose dense range a mixed
 * plan re-evaluated in float-float from its splines, and exactly. */
int pes_plan_work(PesPlan* plan, int64_t B, int64_t* out /* host [6] */, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PESPACE_GB300_H_ */
