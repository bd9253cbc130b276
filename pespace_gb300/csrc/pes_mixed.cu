// Mixed-precision batched path.
//
//  1. sparse stage (float-float on the FP32 pipes, pes_ff.cuh): at n_sparse
//     log-spaced nodes f_j shared by all samples, the phase
//     Phi_s = Psi + 2 pi f k.x0(t_f) and the three TDI channel transfers G_c
//     (response of the unit-phase waveform with the constellation-centre
//     delay factored out), per (sample, detector);
//  2. not-a-knot cubic splines through the nodes (phase solved and stored in
//     float-float, transfer quantities solved in FP32 and stored as FP32
//     coefficients with float-float values), grid tables and node values
//     staged through shared memory;
//  3. dense stage (FP32 bulk): for every bin, h_c = G_c(f) exp(-i (Phi_s(f) +
//     2 pi f t_c)); the phase of each run of <= 32 bins is anchored at the run
//     start (float-float, the fraction of f t_c from integer arithmetic) and
//     advanced in FP32 with exact split products; the residual |d - h|^2 / S
//     is accumulated with compensation, per-block partials are summed in
//     FP64 in a fixed order;
//  4. gradient: the dense stage also accumulates the adjoint moments
//     sum_bins A_q(f) t^p of each spline interval; a transposed spline solve
//     turns them into node adjoints, and one backward pass recomputes the
//     node values with FP32 dual numbers (PhenomD over the mass and spin
//     parameters, the response over the others) and contracts them with the
//     node adjoints (no dense residuals are stored);
//  5. exact bins: far below merger a light system's time-to-coalescence moves
//     so fast with f that the constellation's orbital motion advances by more
//     than kOrbitPhaseMax radians across one node interval; the splines do
//     not resolve that, so each detector's bins below its first resolved
//     interval are evaluated directly (float-float model, residual against
//     the FP64 data, FP32 tangents for the gradient) and the dense stage
//     skips them.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "pes_plan.cuh"

namespace pes {

constexpr int kNodeQ = 7;         // Phi_s, Re/Im G_A, G_E, G_T
constexpr int kChunkMax = 32;     // bins per phase-anchored run (one warp)
constexpr int kMixThreads = 128;  // 4 warps; each warp owns 32 consecutive runs
constexpr int kMoments = 4;       // t^0..t^3
constexpr int kSparseThreads = 128;
// FP32 copies of the shared grid's spline factors, [kGfCount][J]: h, 1/h, lo, up, 1/den, cp.
enum { kGfH = 0, kGfInvH, kGfLo, kGfUp, kGfInvDen, kGfCp, kGfCount };
// Gradient: one pass with FP64 values and FP32 tangents for the 9 parameters
// that enter the node quantities non-trivially; ln D_L (G ~ 1/D_L) and phi_c
// (Phi_s shifts by -2 phi_c) are applied analytically.
constexpr int kMixNT = 9;
constexpr double kOrbitPhaseMax = 0.3;  // rad of yearly orbital phase per node interval
constexpr int kExactBlocks = 4;         // blocks per sample of the exact-bin kernel (heliocentric plans)
constexpr int kExactBlocksGeo = 64;     // with a geocentric detector most inspiral bins are exact
constexpr int kExactThreads = 128;
__device__ __constant__ static const int kSlotParam[kMixNT] = {0, 1, 2, 3, 5, 6, 7, 8, 10};
using GradScalar = DualF<kMixNT>;    // exact bins: FP64 values (phases of 1e6 rad), FP32 tangents

// Plans of several modes (IMRPhenomHM) keep every sparse-grid, spline, anchor,
// kink and midpoint buffer, and the per-sample range arrays nsp, nch, sff,
// cfrac, xbind and xbin, per virtual sample v = s * n_modes + k (sample s,
// mode k); the dense stage sums the modes of a bin before forming its
// residual.  n_modes = 1 (IMRPhenomD): v = s.
struct MixedDev {
  int32_t J;                // nodes
  int32_t n_modes;          // 1 (IMRPhenomD) or kHMModes (IMRPhenomHM)
  const PhenomHMCoef<double>* hm;  // [B] the samples' mode coefficients (IMRPhenomHM plans), else null
  int32_t* vcut;            // [B * n_modes] first bin past the mode's range (its mapped Mf = 0.2, or kcut)
  // Multi-mode plans: each mode's phase is only C1 at its two phase-map
  // corners (Mf = fiP, frP).  The jump of d^2 Psi / dMf^2 there, as
  // Jh max(0, Mf - Mf_c)^2 (Jh half the jump), is removed from the node and
  // midpoint phases before the fit and added back by the run anchors (runs
  // past the corner) or per bin (the run that straddles it).
  float4* pkink;            // [B * n_modes][2] per corner: Mf_c (hi, lo), Jh (hi, lo); null for one mode
  int32_t nchunks;
  int32_t n_det;
  int32_t nblk_dense;
  int32_t nblk_sparse;
  int32_t pad;
  double scale;             // FP32 storage scale of data and model
  const double* node_f;     // [J]
  const TdiFactor* tdn;     // [n_det][J] TDI delay factor at the nodes (prefactor set to 1)
  // float-float copies for the node evaluations on the FP32 pipes
  OrbitFF orbit_ff[PES_MAX_DETECTORS];
  OrbitF orbit_f[PES_MAX_DETECTORS];  // FP32 copies for the derivative passes
  FF scale_ff;
  float scale_f;
  double f_step;            // bin spacing (FP64)
  float4* sff;              // [B][2] per sample: (t_c, M) and (Mf_peak, -) as float-float pairs
  unsigned long long* cfrac;  // [B] fraction of f_step t_c in 64-bit fixed point
  FF fstep_ff;              // bin spacing
  const float2* node_ff;    // [J] node frequencies (hi, lo)
  const float4* tdn_ff;     // [n_det][J] node delay factor D (re hi, re lo, im hi, im lo)
  const int32_t* ch_begin;  // [nchunks] first bin of the run
  const int32_t* ch_len;    // [nchunks]
  const int32_t* ch_iv;     // [nchunks] spline interval of the run
  const float* bin_t;       // [nbins] f_i - f_iv(i)
  float4* runs;             // [B][n_det][nchunks][3] per-run phase anchors (RunPhase, 12 floats)
  // Per (detector, bin) inputs of the dense stage, packed for three 16-byte loads:
  //   part 0: d_A (re, im), d_E (re, im)     part 1: d_T (re, im), w_A, w_E
  //   part 2: w_T, P (re, im), f_i - f_iv(i)
  // (d scaled data, w inverse scaled PSD, 0 off the channel mask; P the TDI
  // generation prefactor)
  float4* pk;               // [n_det][3][nbins]
  float2* dd;               // [n_det][nbins] sum_c |d|^2 / S in FP64, as a float-float pair (hi, lo)
  int32_t* nsp;             // [B] spline intervals of the sample (nodes 0..nsp)
  int32_t* nch;             // [B] runs with a live bin
  int32_t* xbin;            // [B] max over detectors of xbind
  int32_t* xbind;           // [B][n_det] bins [0, xbind) of a detector are evaluated exactly (not splined)
  const int32_t* iv_first;  // [J + 1] first bin of each interval (nbins past the last)
  double omega[PES_MAX_DETECTORS];  // fastest orbital angular frequency of each detector
  int32_t xblocks;          // blocks per sample of the exact-bin kernel
  double* xpart;            // [B][xblocks] exact-bin lnL partials
  double* xgpart;           // [B][xblocks][11] exact-bin gradient partials
  const double* gh;         // [J] node spacing h_i
  const double* ginvh;      // [J] 1 / h_i
  const double* glo;        // [J] reduced not-a-knot system, rows 1..J-2 (first-row elimination included)
  const double* gup;        // [J]
  const double* ginvden;    // [J] 1 / Thomas pivots
  const double* gcp;        // [J] Thomas super-diagonal ratios
  const float* gf;          // [kGfCount][J] FP32 copies of gh, ginvh, glo, gup, ginvden, gcp
  const FF* gff;            // [kGfCount][J] float-float copies of the same
  FF* yv;                   // [B][n_det][7][J] node values (float-float, node fastest)
  double* scr;              // [B][n_det][J][7] spline scratch
  FF* cphi;                 // [B][n_det][J][4] phase spline coefficients (float-float)
  // [B][n_det][J][8] transfer spline coefficients: slots 0-5 (a_hi, b, c, d) of
  // quantities 1..6 in FP32, slots 6-7 the six a - a_hi (the value at the left
  // node in float-float), so one interval is eight 16-byte loads
  float4* cg;
  float* mom;               // [B][n_det][J][7][4] adjoint moments (FP32 warp sums, FP32 atomics)
  float* ybar;              // [B][n_det][J][7] node adjoints (FP32: the derivative passes run in FP32)
  double* part;             // [B][nblk_dense][kPartW] partials: sum |d - h|^2 w (direct form), sum -2 Re(d^* h) w,
                            //   sum 2 Re sum_{k<l} h_k conj(h_l) w (the modes' cross terms; 0 for one mode),
                            //   the rounding estimate (k_refine_select)
  double* gpart;            // [B][n_det][nblk_sparse][11] gradient partials
  void* gblocks;            // [B] SampleBlock<GradScalar>
  double* gdir;             // [B][n_det] direct t_c term of the gradient
  // Amplitude kink at f_peak: the transfer quantities carry C_q max(0, Mf - Mf_peak)^2
  // (C_q = jump/2 * R_q, R_q = G_q(f_peak)/Ahat(f_peak)); it is removed from the
  // node data before the spline fit and added back per bin.
  double* kinkR;            // [B][n_det][6] R_q
  double* kinkC;            // [B][n_det][6] C_q
  float* kinkF;             // [B][n_det][16] Msec f_step, -, C_0..C_5 as float-float (hi x6, lo x6), the
                            //   interval holding the kink point (multi-mode plans, else -1), -
  float* kinkM;             // [B][n_det][12] dense adjoint moments: sum A_q x^2, sum A_q x
  // The split form of the dense sum, sum |d - h|^2 w = sum |d|^2 w - 2 Re sum d^* h w
  // + sum |h|^2 w, for templates far from the data: |d|^2 w from FP64 suffix
  // sums, |h|^2 w from the transfer splines' coefficients against the data's
  // weight moments (the model's squared modulus is a polynomial in t on each
  // interval), so that only the cross term carries per-bin FP32 rounding.
  const FF* wmom;           // [n_det][nbins][3][7] sums over the bins of k's interval j before k of
                            //   u^p W_c (W_c = w_c |P|^2 / scale^2, u = (f - f_j) / h_j; float-float)
  const FF* wtot;           // [n_det][J][3][7] the same over each whole interval
  const double* dsuf;       // [n_det][nbins + 1] sum_{i >= k} sum_c |d_c|^2 w_c (FP64)
  double* wrow;             // [nbins] set-up scratch: one detector's sum_c |d_c|^2 w_c per bin
  float* cgb;               // [B][n_det][J][6] tails b - b_hi of the transfer splines' slope coefficients
  double* hd;               // [B][n_det][kHdOut] per detector's dense range: sum |h|^2 w, sum |d|^2 w, 0,
                            //   and the splines' error estimate of sum |h|^2 w from the exact model at
                            //   the interval midpoints (signed, absolute), 0
  // The splines' error estimate above (and the midpoint corrections) use the
  // exact transfer quantities at the interval midpoints.
  const float2* mid_ff;     // [J] interval midpoints (hi, lo)
  const float4* tdm_ff;     // [n_det][J] TDI delay factor at the midpoints
  FF* ym;                   // [B][n_det][7][J] transfer quantities (rows 0-5, kink removed) and the
                            //   phase (row 6) at the midpoints
  // The splines' error at the midpoints, added back per bin with the shape of
  // the leading error term of cubic interpolation:
  float4* cbump;            // [B][n_det][J][2] delta_0..delta_5, h, 4 / h^2
  // Intervals whose weight |P|^2 / S spikes (a TDI zero where the PSD's own
  // zero does not cancel the prefactor's exactly, e.g. f L = 1 at the top of
  // a 0.1 Hz band): there the midpoint value says nothing about the error at
  // the few bins that carry the weight, so neither the correction nor the
  // split form's error estimate uses it.
  const int32_t* wspike;    // [n_det][J] 1 where max_bin W > kSpikeRatio x mean W over the interval
  int32_t rblocks;          // blocks per sample of the exact re-evaluation
  int32_t refine_all;       // 1: every sample in the domain is re-evaluated (exactly where its spline
                            //   estimate says so, else in float-float)
  double* rpart;            // [B][rblocks] exact dense-range partials of re-evaluated samples
  // How each sample's dense range is re-evaluated, chosen after the dense
  // stage from its FP32 rounding estimate (the dense stage's own sum of
  // |d|^2 |h|^2 w^2) and its splines' error estimate (k_hd): not at all, in
  // float-float from the same splines (rounding: k_dense_ff), or exactly
  // (spline error: k_exact<3>).
  int32_t* rkind;           // [B] kRefineNone, kRefineFF or kRefineExact
  double* fpart;            // [B][nblk_dense] float-float dense-range partials
  // Float-float copies of the FP64 inputs of one bin for k_dense_ff, six rows
  // per detector: d_A, d_E, d_T (re hi, re lo, im hi, im lo; scaled data),
  // (w_A hi, lo, w_E hi, lo), (w_T hi, lo, P re hi, lo), (P im hi, lo, 0, 0)
  // (w the scaled inverse PSD, 0 off the channel mask; P the TDI prefactor).
  float4* xff;              // [n_det][6][nbins]
  // Windows about the T channel's zeros, f = n / L: there T's transfer and its
  // PSD vanish together (S_T has sin^2(2 pi f L) sin^2(pi f L)), so the
  // weight 1 / S_T grows as (f - n/L)^-4 and would amplify the splines'
  // absolute error (FP32 storage, ~1e-7 of the interval's scale) into lnL
  // errors of 1e-2 from a handful of bins.  The kZeroHalf bins on either side
  // of each such frequency in the band are taken out of the dense stage, its
  // split form and its refinements, and evaluated exactly (float-float model,
  // FP64 residual, k_exact<4>; the gradient from FP64 dual numbers,
  // k_zero_grad: FP32 tangents of T cancel there).
  int32_t nzb[PES_MAX_DETECTORS];  // window bins of each detector
  const int32_t* zbin;      // [n_det][kZeroMax] the window bins, ascending
  int32_t zblocks;          // blocks per sample of the window kernels (0: no windows)
  double* zpart;            // [B][zblocks] window lnL partials
  double* zgpart;           // [B][zblocks][11] window gradient partials
  void* zgblocks;           // [B] SampleBlock<Dual<11>> (one-mode plans with windows), else null
};
constexpr int kZeroHalf = 64;   // bins on either side of a T-channel zero
constexpr int kZeroMax = 4096;  // window bins per detector
constexpr int kHdOut = 6;
constexpr int kPartW = 4;  // dense partials per block: direct sum, cross term, modes' cross terms, rounding estimate
constexpr int kRefineNone = 0, kRefineFF = 1, kRefineExact = 2;

// Is bin i of detector d in one of its T-channel zero windows (binary search
// of the ascending window bins)?
__device__ __forceinline__ bool in_zero_window(const MixedDev& M, int d, int64_t i) {
  const int n = M.nzb[d];
  if (n == 0) return false;
  const int32_t* z = M.zbin + (size_t)d * kZeroMax;
  if (i < z[0] || i > z[n - 1]) return false;
  int a = 0, b = n - 1;
  while (a < b) {
    const int m = (a + b) >> 1;
    if (z[m] < i)
      a = m + 1;
    else
      b = m;
  }
  return z[a] == i;
}
constexpr double kSpikeRatio = 8.0;
constexpr int kMomStride = 21;  // moments per bin (and interval) of wmom / wtot
constexpr int kRefineBlocks = 32;  // blocks per sample of the exact re-evaluation

// Error-free transformation: s + e == a + b exactly (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

struct GenArg {
  int32_t gen20[PES_MAX_DETECTORS];
};

struct MixedBuffers {
  MixedDev dev;
  GenArg gen;
  std::vector<void*> allocs;
  // The exact-bin kernels use a few SMs for a long dependent chain each; they
  // run on a side stream beside the sparse/spline/dense stages.
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, xready = nullptr;
  // Second stream of the main sequence: the transfer-spline fit beside the
  // phase fit and the run anchors, the transfer adjoint beside the phase
  // adjoint.
  cudaStream_t aux = nullptr;
  // the gradient pass of the dense stage stages its run inputs through shared
  // memory when they exceed half of L2 (they then stream from DRAM)
  bool stage_grad = false;
  cudaEvent_t ev_nodes = nullptr, ev_tfit = nullptr, ev_dense = nullptr, ev_tadj = nullptr, ev_hd = nullptr, ev_pfit = nullptr,
              ev_kink = nullptr, ev_xgrad = nullptr;
  std::vector<int32_t> zbin_host;  // the zero windows' bins ([n_det][kZeroMax]), for the work report
};

// ------------------------------------------------------------------ sparse stage
// Node values of mode k of a multi-mode (IMRPhenomHM) sample, or of the
// IMRPhenomD model when hm is null: the phase Phi = Psi_k + 2 pi f k.x0 at the
// mode's t(f) and the three channels' transfer of the mode (response of the
// unit-phase mode, centre delay factored out; h_k = A_k e^{-i Psi_k},
// hp = P_k h_k, hc = i C_k h_k).  The orbit, frequency and TDI factors come
// in the scalar types of the caller's pass (float-float for the value
// passes).  kPre applies the TDI generation prefactor Pf (exact bins); nodes
// take it as 1.  The modes continue past their mapped Mf = 0.2 here (smooth
// splines); the dense stage and the exact bins cut them per bin.
template <bool kPre, class T, class O, class Fq>
__device__ __forceinline__ void node_eval_mode(const O& orbit, const Fq& scale, const SampleBlock<T>& b,
                                               const PhenomHMCoef<T>* hm, int k, const Cx<T>& D, const Cx<T>& Pf,
                                               const Fq& f, T y[kNodeQ], bool* live = nullptr) {
  const T Mf = b.wf.Msec * f;
  T amp, psi, tf;
  const T zero = lift<T>(0.0);
  Cx<T> hp, hc;
  if (hm) {
    T f22;
    phenomhm_eval<T>(b.wf, *hm, k, Mf, amp, psi, tf, &f22);
    if (live) *live = val(f22) <= kMfCut;
    amp = amp * scale;
    hp = cx(hm->md[k].P * amp, zero);
    hc = cx(zero, hm->md[k].C * amp);
  } else {
    phenomd_eval<T>(b.wf, Mf, amp, psi, tf);
    if (live) *live = true;
    amp = amp * scale;
    hp = cx(b.wf.pfac * amp, zero);
    hc = cx(zero, -(b.wf.cfac * amp));
  }
  Cx<T> L[6], C[3];
  T kx0;
  single_links_impl<true, T>(orbit, f, hp, hc, tf + b.tc, b.pol, L, &kx0);
  tdi_channels_t<kPre, T>(D, Pf, 1, L, C);
  y[0] = psi + (lift<Fq>(2.0 * kPi) * f) * kx0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    y[1 + 2 * c] = C[c].re;
    y[2 + 2 * c] = C[c].im;
  }
}

// float-float copy of a sample's mode coefficients, written cooperatively
__device__ __forceinline__ void narrow_hm_ff(const PhenomHMCoef<double>& a, PhenomHMCoef<FF>& b) {
  static_assert(sizeof(PhenomHMCoef<FF>) == sizeof(PhenomHMCoef<double>), "FF mode block layout");
  constexpr int nv = (int)(sizeof(PhenomHMCoef<double>) / sizeof(double));
  const double* src = reinterpret_cast<const double*>(&a);
  FF* dst = reinterpret_cast<FF*>(&b);
  for (int j = threadIdx.x; j < nv; j += blockDim.x) dst[j] = ff_from(src[j]);
}
__device__ __forceinline__ void load_hm(const PhenomHMCoef<double>* hm, int64_t s, PhenomHMCoef<double>& out) {
  constexpr int n8 = (int)(sizeof(PhenomHMCoef<double>) / 8);
  const double* src = reinterpret_cast<const double*>(hm + s);
  double* dst = reinterpret_cast<double*>(&out);
  for (int j = threadIdx.x; j < n8; j += blockDim.x) dst[j] = src[j];
}

// FF copy of a sample block (wf, pol, tc converted; cut and status copied),
// written cooperatively by the block's threads.  The two layouts coincide:
// sizeof(FF) == sizeof(double).
__device__ __forceinline__ void narrow_block_ff(const SampleBlock<double>& a, SampleBlock<FF>& b) {
  static_assert(sizeof(SampleBlock<FF>) == sizeof(SampleBlock<double>), "FF block layout");
  static_assert(offsetof(SampleBlock<FF>, fcut) == offsetof(SampleBlock<double>, fcut), "FF block layout");
  constexpr int nv = (int)(offsetof(SampleBlock<double>, fcut) / sizeof(double));  // wf, pol, tc
  const double* src = reinterpret_cast<const double*>(&a);
  FF* dst = reinterpret_cast<FF*>(&b);
  for (int j = threadIdx.x; j < nv; j += blockDim.x) dst[j] = ff_from(src[j]);
  if (threadIdx.x == 0) {
    b.fcut = a.fcut;
    b.kcut = a.kcut;
    b.status = a.status;
    b.pad = 0;
  }
}

// Gradient pass of the exact bins, by the same structure as the backward node
// stage: PhenomD with float-float values and FP32 tangents over the four mass
// and spin parameters (EM), the response per unit amplitude with five (ER:
// T = t(f) + t_c, lambda, sin beta, psi, cos iota).
using EM = Dual<4, float, FF>;
using ER = Dual<5, float, FF>;
struct ExactGradBlock {
  PhenomDCoef<EM> wf;
  Polar<ER> pol;
  ER pfac, cfac;
  FF tc;
  int32_t status;
};

__device__ __forceinline__ void narrow_exact_grad(const SampleBlock<GradScalar>& a, ExactGradBlock& b) {
  constexpr int nwf = (int)(sizeof(PhenomDCoef<GradScalar>) / sizeof(GradScalar));
  constexpr int npol = (int)(sizeof(Polar<GradScalar>) / sizeof(GradScalar));
  static_assert(sizeof(PhenomDCoef<EM>) / sizeof(EM) == nwf, "coefficient block must be an array of scalars");
  static_assert(sizeof(Polar<ER>) / sizeof(ER) == npol, "polarisation block must be an array of scalars");
  const GradScalar* ws = reinterpret_cast<const GradScalar*>(&a.wf);
  EM* wd = reinterpret_cast<EM*>(&b.wf);
  for (int k = threadIdx.x; k < nwf; k += blockDim.x) {
    wd[k].v = ff_from(ws[k].v);
#pragma unroll
    for (int t = 0; t < 4; ++t) wd[k].d[t] = ws[k].d[t];
  }
  const GradScalar* ps = reinterpret_cast<const GradScalar*>(&a.pol);
  ER* pd = reinterpret_cast<ER*>(&b.pol);
  for (int k = threadIdx.x; k < npol; k += blockDim.x) {
    pd[k].v = ff_from(ps[k].v);
    pd[k].d[0] = 0.0f;
    pd[k].d[1] = ps[k].d[5];  // lambda
    pd[k].d[2] = ps[k].d[6];  // sin beta
    pd[k].d[3] = ps[k].d[7];  // psi
    pd[k].d[4] = 0.0f;
  }
  if (threadIdx.x == 0) {
    b.pfac.v = ff_from(a.wf.pfac.v);
    b.cfac.v = ff_from(a.wf.cfac.v);
#pragma unroll
    for (int t = 0; t < 4; ++t) b.pfac.d[t] = b.cfac.d[t] = 0.0f;
    b.pfac.d[4] = a.wf.pfac.d[4];  // cos iota
    b.cfac.d[4] = a.wf.cfac.d[4];
    b.tc = ff_from(a.tc.v);
    b.status = a.status;
  }
}

template <class T>
__device__ __forceinline__ void load_block(const SampleBlock<T>* blocks, int s, SampleBlock<T>& sb) {
  const int n8 = sizeof(SampleBlock<T>) / 8;
  const double* src = reinterpret_cast<const double*>(&blocks[s]);
  double* dst = reinterpret_cast<double*>(&sb);
  for (int j = threadIdx.x; j < n8; j += blockDim.x) dst[j] = src[j];
}

// Kink coefficients per (virtual sample, detector): the amplitude kink of
// the sample's model (IMRPhenomD), or of mode k (IMRPhenomHM: hm_kink).
__global__ void k_kink(PlanDev P, MixedDev M, GenArg G, const SampleBlock<double>* __restrict__ blocks, int64_t B) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= B * M.n_modes * (int64_t)M.n_det) return;
  const int64_t v = t / M.n_det;
  const int d = (int)(t % M.n_det);
  const int64_t s = v / M.n_modes;
  const int k = (int)(v % M.n_modes);
  const SampleBlock<double>& b = blocks[s];
  double* R = M.kinkR + (size_t)t * 6;
  double* C = M.kinkC + (size_t)t * 6;
  float* F = M.kinkF + (size_t)t * 16;
  for (int q = 0; q < 16; ++q) F[q] = 0.0f;
  for (int q = 0; q < 6; ++q) {
    R[q] = 0.0;
    C[q] = 0.0;
  }
  if (b.status != kSampleOk) return;
  const PhenomHMCoef<double>* hm = M.hm ? M.hm + s : nullptr;
  double mf_pk, ahat, jump;
  if (hm)
    hm_kink<double>(b.wf, *hm, k, mf_pk, ahat, jump);
  else {
    mf_pk = b.wf.fpeak;
    amp_peak_jump<double>(b.wf, ahat, jump);
  }
  const double fpk = mf_pk / b.wf.Msec;
  double y[kNodeQ];
  {
    Cx<double> D, Pf;
    tdi_factors(fpk, P.orbit[d].arm_sec, G.gen20[d], D, Pf);
    // the generation prefactor is applied per bin, outside the splines
    node_eval_mode<false, double>(P.orbit[d], M.scale, b, hm, k, D, cx(1.0, 0.0), fpk, y);
  }
  F[0] = (float)(b.wf.Msec * P.f_step);
  F[14] = -1.0f;
  if (hm) {
    // Multi-mode plans carry the kink term in the coefficients of the
    // intervals past the kink point (k_bump): far past the peak C x^2 grows
    // to tens of times the mode's peak amplitude, and adding it back per bin
    // in FP32 lost 1e-5 of the peak model.  Only the interval holding the
    // kink point adds it per bin; its index in F[14].
    int a = 0, z = M.J - 2;  // last interval starting at or below the kink point
    while (a < z) {
      const int mid = (a + z + 1) >> 1;
      if (b.wf.Msec * M.node_f[mid] <= mf_pk) a = mid; else z = mid - 1;
    }
    F[14] = (float)a;
  }
  for (int q = 0; q < 6; ++q) {
    R[q] = y[1 + q] / ahat;
    C[q] = 0.5 * jump * R[q];
    const float hi = (float)C[q];
    F[2 + q] = hi;
    F[8 + q] = (float)(C[q] - (double)hi);
  }
}

// Forward: node values in float-float arithmetic.  grid (ceil(J/128), n_det, B)
// kMid: the six transfer quantities at the midpoints of intervals 0..nsp-1
// instead (the exact model that the splines' error estimates compare with).
template <bool kMid>
__global__ void __launch_bounds__(kSparseThreads) k_sparse_fwd(PlanDev P, MixedDev M, GenArg G,
                                                               const SampleBlock<double>* __restrict__ blocks) {
  __shared__ SampleBlock<double> sb;
  __shared__ SampleBlock<FF> sbf;
  __shared__ PhenomHMCoef<double> hmd;
  __shared__ PhenomHMCoef<FF> hmf;
  const int v = blockIdx.z, d = blockIdx.y;  // virtual sample (sample, mode), detector
  const int s = v / M.n_modes, k = v % M.n_modes;
  load_block(blocks, s, sb);
  if (M.hm) load_hm(M.hm, s, hmd);
  __syncthreads();
  narrow_block_ff(sb, sbf);
  if (M.hm) narrow_hm_ff(hmd, hmf);
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int ns = M.nsp[v];
  if (sb.status != kSampleOk || ns < 3 || j > ns || j >= M.J || (kMid && j >= ns)) return;
  const size_t vd = (size_t)v * M.n_det + d;
  FF y[kNodeQ];
  {
    const float2 fn = kMid ? M.mid_ff[j] : M.node_ff[j];
    const float4 t4 = kMid ? M.tdm_ff[(size_t)d * M.J + j] : M.tdn_ff[(size_t)d * M.J + j];
    const Cx<FF> D = cx(ff_make(t4.x, t4.y), ff_make(t4.z, t4.w));
    node_eval_mode<false, FF>(M.orbit_ff[d], M.scale_ff, sbf, M.hm ? &hmf : nullptr, k, D, D, ff_make(fn.x, fn.y),
                              y);
    const float4 pk = M.sff[2 * v + 1];  // the model's (mode's) amplitude kink point, Mf
    const FF mff = sbf.wf.Msec * ff_make(fn.x, fn.y);
    const FF xk = mff - ff_make(pk.x, pk.y);
    if (M.pkink) {  // the phase's corner terms
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float4 q = M.pkink[2 * v + c];
        const FF xc = mff - ff_make(q.x, q.y);
        if (xc.hi > 0.0f) y[0] = y[0] - ff_make(q.z, q.w) * (xc * xc);
      }
    }
    if (xk.hi > 0.0f) {
      const double* C = M.kinkC + vd * 6;
      const FF x2 = xk * xk;
#pragma unroll
      for (int q = 0; q < 6; ++q) y[1 + q] = y[1 + q] - ff_from(C[q]) * x2;
    }
  }
  if (kMid) {
    FF* out = M.ym + vd * 7 * M.J + j;
#pragma unroll
    for (int q = 0; q < 6; ++q) out[(size_t)q * M.J] = y[1 + q];
    out[(size_t)6 * M.J] = y[0];
    return;
  }
  FF* out = M.yv + vd * kNodeQ * M.J + j;
#pragma unroll
  for (int q = 0; q < kNodeQ; ++q) out[(size_t)q * M.J] = y[q];
}

// Gradient set-up: per sample, the coefficient block with exact FP64
// tangents, stored with FP32 tangents (the exact bins and the backward node
// stage read it).
__global__ void k_setup_grad(PlanDev P, const double* __restrict__ theta, int64_t B,
                             SampleBlock<GradScalar>* __restrict__ out) {
  using TD = Dual<kMixNT, double>;
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  double raw[11];
  for (int j = 0; j < 11; ++j) raw[j] = theta[11 * s + j];
  SampleBlock<GradScalar>& o = out[s];
  if (!theta_in_domain(raw)) {
    o.status = kSampleOutOfDomain;
    return;
  }
  TD th[11];
  for (int j = 0; j < 11; ++j) {
    int slot = -1;
    for (int k = 0; k < kMixNT; ++k)
      if (kSlotParam[k] == j) slot = k;
    th[j] = Seed<TD>::make(raw[j], slot);
  }
  PhenomDCoef<TD> wf;
  phenomd_setup<TD>(th, P.f_ref, wf);
  Polar<TD> pol;
  TD sb = th[7];
  TD cb = dsqrt((1.0 - sb) * (1.0 + sb));
  make_polar<TD>(th[6], sb, cb, th[8], pol);
  static_assert(sizeof(PhenomDCoef<TD>) / sizeof(TD) == sizeof(PhenomDCoef<GradScalar>) / sizeof(GradScalar),
                "coefficient block must be an array of scalars");
  static_assert(sizeof(Polar<TD>) / sizeof(TD) == sizeof(Polar<GradScalar>) / sizeof(GradScalar),
                "polarisation block must be an array of scalars");
  auto narrow = [](const TD* a, GradScalar* b, int n) {
    for (int k = 0; k < n; ++k) {
      b[k].v = a[k].v;
      for (int i = 0; i < kMixNT; ++i) b[k].d[i] = (float)a[k].d[i];
    }
  };
  narrow(reinterpret_cast<const TD*>(&wf), reinterpret_cast<GradScalar*>(&o.wf),
         sizeof(PhenomDCoef<TD>) / sizeof(TD));
  narrow(reinterpret_cast<const TD*>(&pol), reinterpret_cast<GradScalar*>(&o.pol), sizeof(Polar<TD>) / sizeof(TD));
  narrow(&th[10], &o.tc, 1);
  o.status = kSampleOk;
}

// Backward node stage in one pass, by the structure of the node values:
// PhenomD (amplitude A, phase Psi, t(f)) depends on the four mass and spin
// parameters only, and the transfer values are linear in A,
//   y_q = A Y_q(T, lambda, sin beta, psi, cos iota) - C_q x^2,  T = t(f) + t_c,
//   y_0 = Psi + 2 pi f k.x0(T, lambda, sin beta).
// So PhenomD runs with 4 FP32 tangents (GM) and the response, with A = 1,
// with 5 (GR: T, lambda, sin beta, psi, cos iota); the chain rule combines
// them after contracting with the node adjoints W:
//   dL/dm_k  += G_A dA/dm_k + G_T dt/dm_k + W_0 dPsi/dm_k - sum_q W_q R_q dx2h/dm_k
//   dL/dt_c  += G_T,   dL/dr_k += G_r[k]
// with G_A = sum W_q Y_q, G_T = sum W_q A dY_q/dT + W_0 2 pi f dkx0/dT and
// G_r the same for the response parameters.  Same results as carrying all
// nine tangents through the whole evaluation, at about half the work.
using GM = DualS<4>;  // tangent slots 0-3: ln Mc, q, chi_1, chi_2
using GR = DualS<5>;  // T, lambda, sin beta, psi, cos iota

struct BwdBlock {
  PhenomDCoef<GM> wf;
  Polar<GR> pol;
  GR pfac, cfac;
  float tc;
  int status;
};

__global__ void __launch_bounds__(kSparseThreads, 3) k_sparse_bwd_split(PlanDev P, MixedDev M, GenArg G,
                                                                      double wscale) {
  __shared__ BwdBlock sb;
  __shared__ float2 red[kSparseThreads / 32][11];  // per warp: float-float partial sums
  __shared__ double kadd[6][5];                     // dense-side kink terms, added in order to warp 0's sums
  __shared__ int kink_on;
  __shared__ float kR[6];  // the kink coefficients R_q held fixed, narrowed once
  const int s = blockIdx.z, d = blockIdx.y;
  if (threadIdx.x < 6) kR[threadIdx.x] = (float)M.kinkR[((size_t)s * M.n_det + d) * 6 + threadIdx.x];
  {
    // narrow the sample's gradient block (FP64 values, FP32 tangents in slots 0-8)
    const SampleBlock<GradScalar>& g = reinterpret_cast<const SampleBlock<GradScalar>*>(M.gblocks)[s];
    constexpr int nwf = (int)(sizeof(PhenomDCoef<GradScalar>) / sizeof(GradScalar));
    constexpr int npol = (int)(sizeof(Polar<GradScalar>) / sizeof(GradScalar));
    static_assert(sizeof(PhenomDCoef<GM>) / sizeof(GM) == nwf, "coefficient block must be an array of scalars");
    static_assert(sizeof(Polar<GR>) / sizeof(GR) == npol, "polarisation block must be an array of scalars");
    const GradScalar* wsrc = reinterpret_cast<const GradScalar*>(&g.wf);
    GM* wdst = reinterpret_cast<GM*>(&sb.wf);
    for (int k = threadIdx.x; k < nwf; k += blockDim.x) {
      wdst[k].v = (float)wsrc[k].v;
#pragma unroll
      for (int t = 0; t < 4; ++t) wdst[k].d[t] = wsrc[k].d[t];
    }
    const GradScalar* psrc = reinterpret_cast<const GradScalar*>(&g.pol);
    GR* pdst = reinterpret_cast<GR*>(&sb.pol);
    for (int k = threadIdx.x; k < npol; k += blockDim.x) {
      pdst[k].v = (float)psrc[k].v;
      pdst[k].d[0] = 0.0f;
      pdst[k].d[1] = psrc[k].d[5];  // lambda
      pdst[k].d[2] = psrc[k].d[6];  // sin beta
      pdst[k].d[3] = psrc[k].d[7];  // psi
      pdst[k].d[4] = 0.0f;
    }
    if (threadIdx.x == 0) {
      sb.pfac.v = (float)g.wf.pfac.v;
      sb.cfac.v = (float)g.wf.cfac.v;
#pragma unroll
      for (int t = 0; t < 4; ++t) sb.pfac.d[t] = sb.cfac.d[t] = 0.0f;
      sb.pfac.d[4] = g.wf.pfac.d[4];  // cos iota
      sb.cfac.d[4] = g.wf.cfac.d[4];
      sb.tc = (float)g.tc.v;
      sb.status = g.status;
    }
  }
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int ns = M.nsp[s];
  float acc[11];  // this node's contribution (FP32: one node per thread)
#pragma unroll
  for (int k = 0; k < 11; ++k) acc[k] = 0.0f;
  if (sb.status == kSampleOk && ns >= 3 && j <= ns && j < M.J) {
    const float fj = M.node_ff[j].x;
    const float* yb = M.ybar + (((size_t)s * M.n_det + d) * M.J + j) * kNodeQ;
    float W[kNodeQ];
#pragma unroll
    for (int q = 0; q < kNodeQ; ++q) W[q] = yb[q];
    // PhenomD with the mass and spin tangents
    GM amp, psi, tf;
    phenomd_eval<GM>(sb.wf, sb.wf.Msec * fj, amp, psi, tf);
    amp = amp * M.scale_f;
    // response per unit amplitude with the T and sky/orientation tangents
    Cx<GR> Y[3];
    GR kx0;
    {
      GR T = lift<GR>(tf.v + sb.tc);
      T.d[0] = 1.0f;
      const GR zero = lift<GR>(0.0);
      const Cx<GR> hp = cx(sb.pfac, zero), hc = cx(zero, -sb.cfac);
      const float4 t4 = M.tdn_ff[(size_t)d * M.J + j];
      const Cx<GR> D = cx(lift<GR>(t4.x), lift<GR>(t4.z));
      Cx<GR> L[6];
      single_links_impl<true, GR>(M.orbit_f[d], fj, hp, hc, T, sb.pol, L, &kx0);
      tdi_channels_t<false, GR>(D, D, 1, L, Y);
    }
    const float tpf = 6.283185307179586f * fj;
    // contractions over the quantities
    float GA = 0.0f, GT = W[0] * tpf * kx0.d[0], Gr[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) Gr[k] = W[0] * tpf * kx0.d[1 + k];
    float yv[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const GR* yc[2] = {&Y[c].re, &Y[c].im};
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int q = 1 + 2 * c + r;
        const GR& y = *yc[r];
        GA = fmaf(W[q], y.v, GA);
        const float wa = W[q] * amp.v;
        GT = fmaf(wa, y.d[0], GT);
#pragma unroll
        for (int k = 0; k < 4; ++k) Gr[k] = fmaf(wa, y.d[1 + k], Gr[k]);
        yv[2 * c + r] = amp.v * y.v;
      }
    }
    // peak kink removed from the node data: y_q -= R_q x2h, R_q held fixed
    float kx[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const GM xk = sb.wf.Msec * fj - sb.wf.fpeak;
    if (xk.v > 0.0f) {
      GM ahat, jump;
      amp_peak_jump<GM>(sb.wf, ahat, jump);
      const GM x2h = 0.5 * (xk * xk) * jump;
      float WR = 0.0f;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const float Rq = kR[q];
        WR = fmaf(W[1 + q], Rq, WR);
        yv[q] -= Rq * x2h.v;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) kx[k] = WR * x2h.d[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      acc[k] = GA * amp.d[k] + GT * tf.d[k] + W[0] * psi.d[k] - kx[k];  // ln Mc, q, chi_1, chi_2
    acc[5] = Gr[3];   // cos iota
    acc[6] = Gr[0];   // lambda
    acc[7] = Gr[1];   // sin beta
    acc[8] = Gr[2];   // psi
    acc[10] = GT;     // t_c
    float a4 = 0.0f;  // the transfer values scale as 1/D_L
#pragma unroll
    for (int q = 0; q < 6; ++q) a4 = fmaf(-W[1 + q], yv[q], a4);
    acc[4] = a4;
    acc[9] = -2.0f * W[0];  // Phi_s = ... - 2 phi_c
  }
  // block sum: float-float across the warp (FP32 pipe); the FP64 pipe (1/64
  // of the FP32 rate) only in the 11 threads that add the warps' partials
  const int wid = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 11; ++k) {
    float hi = acc[k], lo = 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_down_sync(0xffffffffu, hi, o);
      const float ol = __shfl_down_sync(0xffffffffu, lo, o);
      float th, tl;
      two_sum(hi, oh, th, tl);
      hi = th;
      lo += tl + ol;
    }
    if (l == 0) red[wid][k] = make_float2(hi, lo);
  }
  // dense-side kink term C_q x^2 (x = Msec f - Mf_peak): one thread per (sample, detector)
  if (threadIdx.x == 0) kink_on = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0 && sb.status == kSampleOk && ns >= 3) {
    GM ahat, jump;
    amp_peak_jump<GM>(sb.wf, ahat, jump);
    const double* R = M.kinkR + ((size_t)s * M.n_det + d) * 6;
    const double* C = M.kinkC + ((size_t)s * M.n_det + d) * 6;
    const float* K = M.kinkM + ((size_t)s * M.n_det + d) * 12;
    for (int q = 0; q < 6; ++q) {
      // sum A_q x f = (sum A_q x^2 + Mf_peak sum A_q x) / Msec  (f = (x + Mf_peak) / Msec)
      const double K2 = wscale * K[q], K1 = wscale * K[6 + q];
      const double K1f = (K2 + (double)sb.wf.fpeak.v * K1) / (double)sb.wf.Msec.v;
      for (int k = 0; k < 4; ++k)
        kadd[q][k] = 0.5 * R[q] * K2 * (double)jump.d[k] +
                     2.0 * C[q] * (K1f * (double)sb.wf.Msec.d[k] - K1 * (double)sb.wf.fpeak.d[k]);
      kadd[q][4] = -(C[q] * K2);  // C_q ~ 1/D_L
    }
    kink_on = 1;
  }
  __syncthreads();
  if (threadIdx.x < 11) {
    const int k = threadIdx.x;
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < kSparseThreads / 32; ++w) {
      double v = (double)red[w][k].x + (double)red[w][k].y;
      if (w == 0 && kink_on && k < 5)
        for (int q = 0; q < 6; ++q) v += kadd[q][k];
      x += v;
    }
    M.gpart[(((size_t)s * M.n_det + d) * M.nblk_sparse + blockIdx.x) * 11 + k] = x;
  }
}

// ------------------------------------------------------------------ per-sample ranges
// nsp: intervals 0..nsp-1 cover every live bin (nodes 0..nsp); nch: runs with a
// live bin; xbin: bins below the first interval whose yearly orbital phase
// advance omega |t(f_{j+1}) - t(f_j)| is at most kOrbitPhaseMax (that advance
// falls monotonically with f over the inspiral, so a bisection finds it).
// kPart 0 writes nsp and nch (needed by the sparse stage), kPart 1 xbin (needed
// from the exact bins and the run anchors on), so the bisection can run on the
// side stream.
template <int kPart>
__global__ void k_mixed_ranges(PlanDev P, MixedDev M, const SampleBlock<double>* __restrict__ blocks, int64_t B) {
  // kPart 0: one thread per virtual sample v; kPart 1: one thread per sample
  const int nm = M.n_modes;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (kPart == 0 ? B * nm : B)) return;
  const int64_t s = kPart == 0 ? t / nm : t;
  const int kmode = kPart == 0 ? (int)(t % nm) : 0;
  const SampleBlock<double>& b = blocks[s];
  const PhenomHMCoef<double>* hm = M.hm ? M.hm + s : nullptr;
  // the range's last live bin: the sample's cut, and for mode k of a
  // multi-mode model its mapped Mf = 0.2 (the mode's own cut)
  int64_t kc = b.status == kSampleOk ? b.kcut : 0;
  if (kPart == 0) {
    // the model's (the mode's) amplitude kink point: PhenomD's f_peak, or
    // where the mode's amplitude map turns linear at its mapped f_peak
    const double mfpk = (hm && kmode > 0) ? hm->md[kmode].frA : b.wf.fpeak;
    const FF tcf = ff_from(b.tc), msf = ff_from(b.wf.Msec), fpf = ff_from(mfpk);
    M.sff[2 * t] = make_float4(tcf.hi, tcf.lo, msf.hi, msf.lo);
    M.sff[2 * t + 1] = make_float4(fpf.hi, fpf.lo, 0.0f, 0.0f);
    // f t_c = (k0 + k) c, c = f_step t_c: its fraction is (k0 + k) frac(c) mod 1
    const double cyc = M.f_step * b.tc;
    const double rs = (cyc - floor(cyc)) * 18446744073709551616.0;  // 2^64
    M.cfrac[t] = (rs >= 0.0 && rs < 18446744073709551616.0) ? (unsigned long long)rs : 0ull;
    if (hm && kc > 0) {
      // first bin whose mapped frequency passes Mf = 0.2 (the linear map, as
      // the mode's model evaluates it past its amplitude corner)
      const double Rk = hm->md[kmode].Rholm;
      int64_t lo = 0, hi = kc;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        const double Mf = b.wf.Msec * ((double)(P.k0 + mid) * P.f_step);
        if ((kmode == 0 ? Mf : Rk * Mf) <= kMfCut) lo = mid + 1; else hi = mid;
      }
      kc = lo;
    }
    M.vcut[t] = (int32_t)kc;
    if (M.pkink) {
      // the phase's second-derivative jumps at the mode's phase-map corners:
      // one-sided second differences of dPsi/dMf, 1e-6 of Mf_c apart
      float4* pk = M.pkink + 2 * t;
      for (int c = 0; c < 2; ++c) {
        double jh = 0.0, mfc = 1.0;
        if (b.status == kSampleOk && hm) {
          const HMMode<double>& md = hm->md[kmode];
          const int m = kHMlm[kmode][1];
          mfc = c == 0 ? md.fiP : md.frP;
          const double e = 1e-6 * mfc;
          auto dps = [&](double x) {
            double ps, dp;
            hm_phase<double>(b.wf, md, m, x, ps, dp);
            return dp;
          };
          const double right = (dps(mfc + 2.0 * e) - dps(mfc + e)) / e;
          const double left = (dps(mfc - e) - dps(mfc - 2.0 * e)) / e;
          jh = 0.5 * (right - left);
        }
        const FF a = ff_from(mfc), q = ff_from(jh);
        pk[c] = make_float4(a.hi, a.lo, q.hi, q.lo);
      }
    }
  }
  int ns = 0, nc = 0, xb = 0;
  if (kc > 0) {
    const int64_t last = kc - 1;
    int lo = 0, hi = M.nchunks - 1;  // last run whose first bin is <= last
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (M.ch_begin[mid] <= last) lo = mid; else hi = mid - 1;
    }
    nc = lo + 1;
    ns = M.ch_iv[lo] + 1;
    if (ns < 3) ns = 3;
    if (ns > M.J - 1) ns = M.J - 1;
    if (kPart == 0) {
      M.nsp[t] = ns;
      M.nch[t] = nc;
      return;
    }
    for (int d = 0; d < M.n_det; ++d) {
      int xbd = 0;
      // the exact range: the largest over the modes (each mode's own t(f))
      for (int k = 0; k < nm; ++k) {
        auto tfk = [&](int j) {
          double a, ps, tt;
          const double Mf = b.wf.Msec * M.node_f[j];
          if (hm)
            phenomhm_eval<double>(b.wf, *hm, k, Mf, a, ps, tt, nullptr);
          else
            phenomd_eval<double>(b.wf, Mf, a, ps, tt);
          return tt;
        };
        auto unresolved = [&](int j) { return M.omega[d] * fabs(tfk(j + 1) - tfk(j)) > kOrbitPhaseMax; };
        if (unresolved(0)) {
          int lo2 = 0, hi2 = ns - 1;  // last unresolved interval
          while (lo2 < hi2) {
            int mid = (lo2 + hi2 + 1) >> 1;
            if (unresolved(mid)) lo2 = mid; else hi2 = mid - 1;
          }
          const int64_t first = M.iv_first[lo2 + 1];
          const int x = (int)(first < kc ? first : kc);
          xbd = x > xbd ? x : xbd;
        }
      }
      for (int k = 0; k < nm; ++k) M.xbind[(s * nm + k) * M.n_det + d] = xbd;
      xb = xbd > xb ? xbd : xb;
    }
  } else if (kPart == 1) {
    for (int d = 0; d < M.n_det; ++d)
      for (int k = 0; k < nm; ++k) M.xbind[(s * nm + k) * M.n_det + d] = 0;
  }
  if (kPart == 0) {
    M.nsp[t] = ns;
    M.nch[t] = nc;
  } else {
    for (int k = 0; k < nm; ++k) M.xbin[s * nm + k] = xb;
  }
}

// ------------------------------------------------------------------ splines
// Not-a-knot cubic spline through nodes 0..n (n >= 3).  Unknowns: second
// derivatives m_1..m_{n-1} (m_0 and m_n eliminated with the not-a-knot
// conditions).  Row i: lo_i m_{i-1} + di_i m_i + up_i m_{i+1} = 6 (D_i - D_{i-1}).
__device__ __forceinline__ void nak_row(const double* f, int n, int i, double& lo, double& di, double& up) {
  const double h0 = f[i] - f[i - 1], h1 = f[i + 1] - f[i];
  lo = h0;
  di = 2.0 * (h0 + h1);
  up = h1;
  if (i == 1) {  // m_0 = ((h0 + h1) m_1 - h0 m_2) / h1
    di += h0 * (h0 + h1) / h1;
    up -= h0 * h0 / h1;
    lo = 0.0;
  }
  if (i == n - 1) {  // m_n = ((h_{n-2} + h_{n-1}) m_{n-1} - h_{n-1} m_{n-2}) / h_{n-2}
    di += h1 * (h0 + h1) / h0;
    lo -= h1 * h1 / h0;
    up = 0.0;
  }
}

__device__ __forceinline__ void nak_ends(const double* f, int n, double m1, double m2, double mn1, double mn2,
                                         double& m0, double& mn) {
  const double h0 = f[1] - f[0], h1 = f[2] - f[1];
  m0 = ((h0 + h1) * m1 - h0 * m2) / h1;
  const double ha = f[n - 1] - f[n - 2], hb = f[n] - f[n - 1];
  mn = ((ha + hb) * mn1 - hb * mn2) / ha;
}

// The two recurrences of a tridiagonal solve, x_i = alpha_i x_{i-1} + beta_i,
// are split over the 32 lanes of a warp: each lane runs its segment of rows
// from 0 to get the segment's affine map x_in -> A x_in + B, a warp scan of
// those maps gives the exact value entering every segment, and the lane then
// reruns its segment from that value.  `reverse` scans from lane 31 down.
// Warp shuffles for the spline scalars (float, double, float-float).
__device__ __forceinline__ float warp_shfl_up(float x, int o) { return __shfl_up_sync(0xffffffffu, x, o); }
__device__ __forceinline__ float warp_shfl_down(float x, int o) { return __shfl_down_sync(0xffffffffu, x, o); }
__device__ __forceinline__ double warp_shfl_up(double x, int o) { return __shfl_up_sync(0xffffffffu, x, o); }
__device__ __forceinline__ double warp_shfl_down(double x, int o) { return __shfl_down_sync(0xffffffffu, x, o); }
__device__ __forceinline__ FF warp_shfl_up(const FF& x, int o) {
  return ff_make(__shfl_up_sync(0xffffffffu, x.hi, o), __shfl_up_sync(0xffffffffu, x.lo, o));
}
__device__ __forceinline__ FF warp_shfl_down(const FF& x, int o) {
  return ff_make(__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o));
}

template <class R>
__device__ __forceinline__ R segment_carry_in(R A, R B, bool reverse) {
  const int lane = threadIdx.x & 31;
  const int pos = reverse ? 31 - lane : lane;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const R Ap = reverse ? warp_shfl_down(A, o) : warp_shfl_up(A, o);
    const R Bp = reverse ? warp_shfl_down(B, o) : warp_shfl_up(B, o);
    if (pos >= o) {
      B = A * Bp + B;
      A = A * Ap;
    }
  }
  const R prev = reverse ? warp_shfl_down(B, 1) : warp_shfl_up(B, 1);
  return pos == 0 ? lift<R>(0.0) : prev;
}


constexpr int kSplineThreads = kNodeQ * 32;  // one warp per quantity, one block per (sample, detector)

// Transfer quantities (q >= 1) of the fit: slopes and right-hand sides in FP64
// from the FP64 node values (their differences cancel), the tridiagonal solve
// in FP32 (these coefficients are stored in FP32), the left value as a
// float-float pair.  Scratch per (node, quantity): (rhs | d' | m, slope).
__device__ __forceinline__ void spline_fit_transfer(const MixedDev& M, int64_t sd, int q, int n) {
  const int lane = threadIdx.x & 31;
  const FF* yq = M.yv + ((size_t)sd * kNodeQ + q) * M.J;
  auto y = [&](int i) { return ff_to(yq[i]); };
  float2* S = reinterpret_cast<float2*>(M.scr + (size_t)sd * M.J * kNodeQ + q);
  const float* fh = M.gf + (size_t)kGfH * M.J;
  const float* fih = M.gf + (size_t)kGfInvH * M.J;
  const float* flo = M.gf + (size_t)kGfLo * M.J;
  const float* fid = M.gf + (size_t)kGfInvDen * M.J;
  const float* fcp = M.gf + (size_t)kGfCp * M.J;
  const int seg = (n + 31) >> 5;
  const int i0 = min(n, lane * seg), i1 = min(n, i0 + seg);
  const int r0 = max(1, i0), r1 = i1;
  if (i0 < i1) {
    double sp = (i0 >= 1) ? (y(i0) - y(i0 - 1)) * M.ginvh[i0 - 1] : 0.0;
    for (int i = i0; i < i1; ++i) {
      const double sl = (y(i + 1) - y(i)) * M.ginvh[i];
      S[i * kNodeQ] = make_float2(i >= 1 ? (float)(6.0 * (sl - sp)) : 0.0f, (float)sl);
      sp = sl;
    }
  }
  double lo_d, di_d, up_d;
  nak_row(M.node_f, n, n - 1, lo_d, di_d, up_d);
  const float lo_l = (float)lo_d;
  const float iden_l = (float)(1.0 / (di_d - lo_d * M.gcp[n - 2]));
  float A = 1.0f, x = 0.0f;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r0; i < r1; ++i) {
      const bool last = i == n - 1;
      const float l = last ? lo_l : flo[i];
      const float id = last ? iden_l : fid[i];
      float2 v = S[i * kNodeQ];
      x = (v.x - l * x) * id;
      if (pass == 0) {
        A = -l * id * A;
      } else {
        v.x = x;
        S[i * kNodeQ] = v;
      }
    }
    if (pass == 0) x = segment_carry_in<float>(A, x, false);
  }
  A = 1.0f;
  x = 0.0f;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r1 - 1; i >= r0; --i) {
      const float c = (i == n - 1) ? 0.0f : fcp[i];
      float2 v = S[i * kNodeQ];
      x = v.x - c * x;
      if (pass == 0) {
        A = -c * A;
      } else {
        v.x = x;
        S[i * kNodeQ] = v;
      }
    }
    if (pass == 0) x = segment_carry_in<float>(A, x, true);
  }
  __syncwarp();
  const float h0 = fh[0], h1 = fh[1], ha = fh[n - 2], hb = fh[n - 1];
  const float m0 = ((h0 + h1) * S[1 * kNodeQ].x - h0 * S[2 * kNodeQ].x) / h1;
  const float mn = ((ha + hb) * S[(n - 1) * kNodeQ].x - hb * S[(n - 2) * kNodeQ].x) / ha;
  if (i0 >= i1) return;
  float mi = (i0 == 0) ? m0 : S[i0 * kNodeQ].x;
  for (int i = i0; i < i1; ++i) {
    const float mj = (i + 1 == n) ? mn : S[(i + 1) * kNodeQ].x;
    const float sl = S[i * kNodeQ].y;
    (void)sl;
    // b = slope - h (2 m_i + m_j) / 6 with the FP64 slope: stored as FP32 head and tail
    const double bd = (y(i + 1) - y(i)) * M.ginvh[i] - (double)(fh[i] * (2.0f * mi + mj) * (1.0f / 6.0f));
    const float bc = (float)bd;
    const float cc = 0.5f * mi;
    const float dc = (mj - mi) * fih[i] * (1.0f / 6.0f);
    const FF a = yq[i];
    M.cg[((size_t)sd * M.J + i) * 8 + (q - 1)] = make_float4(a.hi, bc, cc, dc);
    reinterpret_cast<float*>(M.cg + ((size_t)sd * M.J + i) * 8 + 6)[q - 1] = a.lo;
    M.cgb[((size_t)sd * M.J + i) * 6 + (q - 1)] = (float)(bd - (double)bc);
    mi = mj;
  }
}

// Transfer quantities (q >= 1) of the adjoint: right-hand sides from the FP64
// moments in FP64, the transposed solve and the node adjoints in FP32.
__device__ __forceinline__ void spline_adjoint_transfer(const MixedDev& M, int64_t sd, int q, int n, double wscale) {
  const int lane = threadIdx.x & 31;
  const float* mom = M.mom + (size_t)sd * M.J * kNodeQ * kMoments + (size_t)q * kMoments;
  float2* X = reinterpret_cast<float2*>(M.scr + (size_t)sd * M.J * kNodeQ + q);
  float* yb = M.ybar + (size_t)sd * M.J * kNodeQ + q;
  const float* fih = M.gf + (size_t)kGfInvH * M.J;
  const float* flo = M.gf + (size_t)kGfLo * M.J;
  const float* fup = M.gf + (size_t)kGfUp * M.J;
  const float* fid = M.gf + (size_t)kGfInvDen * M.J;
  const int seg = (n + 31) >> 5;
  const int i0 = min(n, lane * seg), i1 = min(n, i0 + seg);
  const int r0 = max(1, i0), r1 = i1;
  auto mm = [&](int i, int p) { return wscale * mom[(size_t)i * kNodeQ * kMoments + p]; };
  auto mbar_left = [&](int i) {
    const double h = M.gh[i], ih = M.ginvh[i];
    return -h * mm(i, 1) * (1.0 / 3.0) + 0.5 * mm(i, 2) - mm(i, 3) * ih * (1.0 / 6.0);
  };
  auto mbar_right = [&](int i) {
    const double h = M.gh[i], ih = M.ginvh[i];
    return -h * mm(i, 1) * (1.0 / 6.0) + mm(i, 3) * ih * (1.0 / 6.0);
  };
  {
    const double mb0 = mbar_left(0), mbn = mbar_right(n - 1);
    const double h0 = M.gh[0], h1 = M.gh[1], ha = M.gh[n - 2], hb = M.gh[n - 1];
    for (int i = r0; i < r1; ++i) {
      double v = mbar_right(i - 1) + mbar_left(i);
      if (i == 1) v += mb0 * (h0 + h1) / h1;
      if (i == 2) v -= mb0 * h0 / h1;
      if (i == n - 1) v += mbn * (ha + hb) / ha;
      if (i == n - 2) v -= mbn * hb / ha;
      X[i * kNodeQ] = make_float2((float)v, 0.0f);
    }
  }
  double lo_d, di_d, up_d;
  nak_row(M.node_f, n, n - 1, lo_d, di_d, up_d);
  const float lo_l = (float)lo_d;
  const float iden_l = (float)(1.0 / (di_d - lo_d * M.gcp[n - 2]));
  float A = 1.0f, x = 0.0f;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r0; i < r1; ++i) {
      const float sub = (i > 1) ? fup[i - 1] : 0.0f;
      const float id = (i == n - 1) ? iden_l : fid[i];
      float2 v = X[i * kNodeQ];
      x = (v.x - sub * x) * id;
      if (pass == 0) {
        A = -sub * id * A;
      } else {
        v.x = x;
        X[i * kNodeQ] = v;
      }
    }
    if (pass == 0) x = segment_carry_in<float>(A, x, false);
  }
  A = 1.0f;
  x = 0.0f;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r1 - 1; i >= r0; --i) {
      const float c = (i == n - 1) ? 0.0f : ((i + 1 == n - 1) ? lo_l : flo[i + 1]) * fid[i];
      float2 v = X[i * kNodeQ];
      x = v.x - c * x;
      if (pass == 0) {
        A = -c * A;
      } else {
        v.x = x;
        X[i * kNodeQ] = v;
      }
    }
    if (pass == 0) x = segment_carry_in<float>(A, x, true);
  }
  __syncwarp();
  auto rb = [&](int i) { return (i >= 1 && i <= n - 1) ? X[i * kNodeQ].x : 0.0f; };
  if (i0 < i1) {
    float rcur = rb(i0);
    float dprev = 0.0f;
    if (i0 > 0) dprev = ((float)mm(i0 - 1, 1) + 6.0f * (rb(i0 - 1) - rcur)) * fih[i0 - 1];
    for (int i = i0; i < i1; ++i) {
      const float rnext = rb(i + 1);
      const float Db = (float)mm(i, 1) + 6.0f * (rcur - rnext);
      yb[i * kNodeQ] = dprev + (float)mm(i, 0) - Db * fih[i];
      dprev = Db * fih[i];
      rcur = rnext;
    }
    if (i1 == n) yb[n * kNodeQ] = dprev;
  }
  for (int i = n + 1 + lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
}

// Fit for grids of more than 64 x 32 intervals (segments in global scratch):
// warp per (sample, detector, quantity); lane l owns intervals and rows
// [l*seg, (l+1)*seg) of the sample's n intervals.  Rows 1..n-2 use the shared
// grid's precomputed Thomas factors, row n-1 the sample's not-a-knot end row.
__global__ void __launch_bounds__(kSplineThreads) k_spline_fit_wide(MixedDev M) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sd = blockIdx.x;
  const int64_t s = sd / M.n_det;
  const int n = M.nsp[s];
  if (n < 3) return;
  if (q > 0) {
    spline_fit_transfer(M, sd, q, n);
    return;
  }
  const double* f = M.node_f;
  const FF* yq = M.yv + ((size_t)sd * kNodeQ + q) * M.J;
  auto y = [&](int i) { return ff_to(yq[i]); };
  double* S = M.scr + (size_t)sd * M.J * kNodeQ + q;       // d' then m
  const int seg = (n + 31) >> 5;
  const int i0 = min(n, lane * seg), i1 = min(n, i0 + seg);  // intervals [i0, i1)
  const int r0 = max(1, i0), r1 = i1;                          // rows [r0, r1), all <= n - 1
  double lo_l, di_l, up_l;
  nak_row(f, n, n - 1, lo_l, di_l, up_l);
  const double iden_l = 1.0 / (di_l - lo_l * M.gcp[n - 2]);
  // forward elimination d'_i = (r_i - lo_i d'_{i-1}) / den_i
  double A = 1.0, x = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    if (r0 < r1) {
      double sp = (y(r0) - y(r0 - 1)) * M.ginvh[r0 - 1];
      for (int i = r0; i < r1; ++i) {
        const double sl = (y(i + 1) - y(i)) * M.ginvh[i];
        const double r = 6.0 * (sl - sp);
        sp = sl;
        const bool last = i == n - 1;
        const double l = last ? lo_l : M.glo[i];
        const double id = last ? iden_l : M.ginvden[i];
        x = (r - l * x) * id;
        if (pass == 0) A = -l * id * A;
        else S[i * kNodeQ] = x;
      }
    }
    if (pass == 0) x = segment_carry_in<double>(A, x, false);
  }
  // back substitution m_i = d'_i - cp_i m_{i+1}  (m_{n-1} = d'_{n-1})
  __syncwarp();
  A = 1.0;
  x = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r1 - 1; i >= r0; --i) {
      const double c = (i == n - 1) ? 0.0 : M.gcp[i];
      x = S[i * kNodeQ] - c * x;
      if (pass == 0) A = -c * A;
      else S[i * kNodeQ] = x;
    }
    if (pass == 0) x = segment_carry_in<double>(A, x, true);
  }
  __syncwarp();
  double m0, mn;
  nak_ends(f, n, S[1 * kNodeQ], S[2 * kNodeQ], S[(n - 1) * kNodeQ], S[(n - 2) * kNodeQ], m0, mn);
  if (i0 >= i1) return;
  double mi = (i0 == 0) ? m0 : S[i0 * kNodeQ];
  double a = y(i0);
  for (int i = i0; i < i1; ++i) {
    const double mj = (i + 1 == n) ? mn : S[(i + 1) * kNodeQ];
    const double h = M.gh[i];
    const double an = y(i + 1);
    const double bc = (an - a) * M.ginvh[i] - h * (2.0 * mi + mj) * (1.0 / 6.0);
    const double cc = 0.5 * mi;
    const double dc = (mj - mi) * M.ginvh[i] * (1.0 / 6.0);
    if (q == 0) {
      FF* o = M.cphi + ((size_t)sd * M.J + i) * 4;
      o[0] = yq[i];
      o[1] = ff_from(bc);
      o[2] = ff_from(cc);
      o[3] = ff_from(dc);
    } else {
      const float ahi = (float)a;
      M.cg[((size_t)sd * M.J + i) * 8 + (q - 1)] = make_float4(ahi, (float)bc, (float)cc, (float)dc);
      reinterpret_cast<float*>(M.cg + ((size_t)sd * M.J + i) * 8 + 6)[q - 1] = (float)(a - (double)ahi);
    }
    mi = mj;
    a = an;
  }
}

// Transpose of the fit: interval coefficient adjoints (the dense moments,
// times wscale) -> node adjoints ybar; also the direct t_c term (q == 0).
// Same warp decomposition as the fit.
__global__ void __launch_bounds__(kSplineThreads) k_spline_adjoint_wide(MixedDev M, double wscale) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sd = blockIdx.x;
  const int64_t s = sd / M.n_det;
  const int n = M.nsp[s];
  float* yb = M.ybar + (size_t)sd * M.J * kNodeQ + q;  // yb[i * kNodeQ]
  if (n < 3) {
    for (int i = lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
    if (q == 0 && lane == 0) M.gdir[sd] = 0.0;
    return;
  }
  if (q > 0) {
    spline_adjoint_transfer(M, sd, q, n, wscale);
    return;
  }
  const double* f = M.node_f;
  const float* mom = M.mom + (size_t)sd * M.J * kNodeQ * kMoments + (size_t)q * kMoments;  // + i*7*4
  double* X = M.scr + (size_t)sd * M.J * kNodeQ + q;  // z, then rbar
  const int seg = (n + 31) >> 5;
  const int i0 = min(n, lane * seg), i1 = min(n, i0 + seg);
  const int r0 = max(1, i0), r1 = i1;
  auto mm = [&](int i, int p) { return wscale * mom[(size_t)i * kNodeQ * kMoments + p]; };
  // mbar_i = (interval i-1 part) + (interval i part)
  auto mbar_left = [&](int i) {  // from interval i (to node i)
    const double h = M.gh[i], ih = M.ginvh[i];
    return -h * mm(i, 1) * (1.0 / 3.0) + 0.5 * mm(i, 2) - mm(i, 3) * ih * (1.0 / 6.0);
  };
  auto mbar_right = [&](int i) {  // from interval i (to node i + 1)
    const double h = M.gh[i], ih = M.ginvh[i];
    return -h * mm(i, 1) * (1.0 / 6.0) + mm(i, 3) * ih * (1.0 / 6.0);
  };
  const double mb0 = mbar_left(0), mbn = mbar_right(n - 1);
  const double h0 = M.gh[0], h1 = M.gh[1], ha = M.gh[n - 2], hb = M.gh[n - 1];
  auto xrow = [&](int i) {  // right-hand side of row i (1..n-1) after the end eliminations
    double v = mbar_right(i - 1) + mbar_left(i);
    if (i == 1) v += mb0 * (h0 + h1) / h1;
    if (i == 2) v -= mb0 * h0 / h1;
    if (i == n - 1) v += mbn * (ha + hb) / ha;
    if (i == n - 2) v -= mbn * hb / ha;
    return v;
  };
  double lo_l, di_l, up_l;
  nak_row(f, n, n - 1, lo_l, di_l, up_l);
  const double iden_l = 1.0 / (di_l - lo_l * M.gcp[n - 2]);
  // U^T z = mbar: z_i = (x_i - up_{i-1} z_{i-1}) / den_i
  double A = 1.0, x = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r0; i < r1; ++i) {
      const double sub = (i > 1) ? M.gup[i - 1] : 0.0;
      const double id = (i == n - 1) ? iden_l : M.ginvden[i];
      x = (xrow(i) - sub * x) * id;
      if (pass == 0) A = -sub * id * A;
      else X[i * kNodeQ] = x;
    }
    if (pass == 0) x = segment_carry_in<double>(A, x, false);
  }
  __syncwarp();
  // L^T rbar = z: rbar_i = z_i - (lo_{i+1} / den_i) rbar_{i+1}
  A = 1.0;
  x = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = r1 - 1; i >= r0; --i) {
      const double c = (i == n - 1) ? 0.0 : ((i + 1 == n - 1) ? lo_l : M.glo[i + 1]) * M.ginvden[i];
      x = X[i * kNodeQ] - c * x;
      if (pass == 0) A = -c * A;
      else X[i * kNodeQ] = x;
    }
    if (pass == 0) x = segment_carry_in<double>(A, x, true);
  }
  __syncwarp();
  // node adjoints: ybar_i = Dbar_{i-1}/h_{i-1} + wscale mm0_i - Dbar_i/h_i,
  // Dbar_i = wscale mm1_i + 6 (rbar_i - rbar_{i+1}); direct t_c term
  auto rb = [&](int i) { return (i >= 1 && i <= n - 1) ? X[i * kNodeQ] : 0.0; };
  double gd = 0.0;
  if (i0 < i1) {
    double rcur = rb(i0);
    double dprev = 0.0;
    if (i0 > 0) dprev = (mm(i0 - 1, 1) + 6.0 * (rb(i0 - 1) - rcur)) * M.ginvh[i0 - 1];
    for (int i = i0; i < i1; ++i) {
      const double rnext = rb(i + 1);
      const double Db = mm(i, 1) + 6.0 * (rcur - rnext);
      yb[i * kNodeQ] = (float)(dprev + mm(i, 0) - Db * M.ginvh[i]);
      dprev = Db * M.ginvh[i];
      rcur = rnext;
      if (q == 0) gd += 2.0 * kPi * (f[i] * mom[(size_t)i * kNodeQ * kMoments] + mom[(size_t)i * kNodeQ * kMoments + 1]);
    }
    if (i1 == n) yb[n * kNodeQ] = (float)dprev;
  }
  for (int i = n + 1 + lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
  if (q == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gd += __shfl_xor_sync(0xffffffffu, gd, o);
    if (lane == 0) M.gdir[sd] = wscale * gd;
  }
}

// Register-segment versions (n <= 64 x 32 intervals; segments of 32 rows for
// the default grid of 1024 nodes, of 64 rows up to 2049 nodes): each
// lane keeps its segment's rows in registers (fully unrolled, predicated
// loops), so the recurrences wait on arithmetic only.  Phase (q == 0) in FP64,
// transfer quantities in FP32 with FP64 slopes and right-hand sides.
constexpr int kSegMax = 64;  // longest register segment (grids of up to 64 x 32 intervals)

// Register segment length for a grid of J nodes (0: use the global-scratch kernels).
inline int spline_seg(int J) { return J <= 32 * 32 + 1 ? 32 : (J <= kSegMax * 32 + 1 ? kSegMax : 0); }

template <class R>
__device__ __forceinline__ const R* spline_factor(const MixedDev& M, int which) {
  if constexpr (std::is_same<R, FF>::value) {
    return M.gff + (size_t)which * M.J;
  } else if constexpr (sizeof(R) == 8) {
    switch (which) {
      case kGfH: return reinterpret_cast<const R*>(M.gh);
      case kGfInvH: return reinterpret_cast<const R*>(M.ginvh);
      case kGfLo: return reinterpret_cast<const R*>(M.glo);
      case kGfUp: return reinterpret_cast<const R*>(M.gup);
      case kGfInvDen: return reinterpret_cast<const R*>(M.ginvden);
      default: return reinterpret_cast<const R*>(M.gcp);
    }
  } else {
    return reinterpret_cast<const R*>(M.gf + (size_t)which * M.J);
  }
}

// Register-segment fit, staged through shared memory.  Each warp solves one
// (sample, detector, quantity) system; lane l owns rows [l seg, (l+1) seg).
// Those lane-strided accesses go to shared memory only: the block first
// copies the shared grid's factor tables and each warp its system's node
// values with coalesced loads (rows padded by one slot per 32, so that the
// lane-strided reads are free of bank conflicts for seg = 32).
// R = FF for the phase (q == 0), float for the transfer quantities; slopes
// and right-hand sides from the float-float node values in FF.
template <class R> __device__ __forceinline__ R ff_to_r(const FF& x);
template <> __device__ __forceinline__ float ff_to_r<float>(const FF& x) { return x.hi; }
template <> __device__ __forceinline__ FF ff_to_r<FF>(const FF& x) { return x; }

constexpr int kFitWarps = 4;  // systems per block of the staged fit
__host__ __device__ __forceinline__ int fit_pad(int i) { return i + (i >> 5); }
__host__ __device__ __forceinline__ int fit_rows(int J) { return fit_pad(J) + 1; }

// dynamic shared memory of one staged-fit block: five R tables (h, 1/h, lo,
// 1/den, cp), the FF 1/h table for the slopes (the R table itself for R = FF),
// then per warp the node values and the four end-row values.
// Grids of more than 32 x 32 intervals leave the tables in global memory
// (staging them would leave room for one block per SM).
template <class R, bool kStageTables>
__host__ __device__ __forceinline__ size_t fit_smem_bytes(int J) {
  const size_t rows = (size_t)fit_rows(J);
  const size_t tables =
      kStageTables ? 5 * rows * sizeof(R) + (std::is_same<R, FF>::value ? 0 : rows * sizeof(FF)) : 0;
  return ((tables + 15) & ~(size_t)15) + (size_t)kFitWarps * (rows * sizeof(FF) + 4 * sizeof(FF));
}

template <int kSeg, class R, bool kStageTables>
__device__ __forceinline__ void spline_fit_staged(const MixedDev& M, int64_t sd, int q, int n, const R* t_h,
                                                  const R* t_ih, const R* t_lo, const R* t_id, const R* t_cp,
                                                  const FF* t_gih, const FF* y, R* smem4) {
  const int lane = threadIdx.x & 31;
  auto tp = [](int i) { return kStageTables ? fit_pad(i) : i; };
  // staged: segments of 32 rows whatever n (lanes past n idle), which keeps
  // the lane-strided shared-memory reads free of bank conflicts
  const int seg = kStageTables ? 32 : (n + 31) >> 5;
  const int i0 = min(n, lane * seg), cnt = min(n, i0 + seg) - i0;
  double lo_d, di_d, up_d;
  nak_row(M.node_f, n, n - 1, lo_d, di_d, up_d);
  const R lo_l = lift<R>(lo_d), iden_l = lift<R>(1.0 / (di_d - lo_d * M.gcp[n - 2]));
  const R zero = lift<R>(0.0);
  // right-hand sides 6 (slope_i - slope_{i-1}) of rows i0 + k
  R x[kSeg];
  {
    FF yc = y[fit_pad(i0)];
    FF sp = (i0 >= 1) ? (yc - y[fit_pad(i0 - 1)]) * t_gih[tp(i0 - 1)] : ff_make(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < kSeg; ++k) {
      x[k] = zero;
      if (k < cnt) {
        const int i = i0 + k;
        const FF yn = y[fit_pad(i + 1)];
        const FF sl = (yn - yc) * t_gih[tp(i)];
        if (i >= 1) x[k] = ff_to_r<R>(ff_mulf(sl - sp, 6.0f));
        sp = sl;
        yc = yn;
      }
    }
  }
  // forward elimination (rows 1..n-1)
  R A = lift<R>(1.0), v = zero;
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const bool last = i == n - 1;
      const R l = last ? lo_l : t_lo[tp(i)], id = last ? iden_l : t_id[tp(i)];
      v = (x[k] - l * v) * id;
      A = -(l * id) * A;
    }
  }
  v = segment_carry_in<R>(A, v, false);
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const bool last = i == n - 1;
      const R l = last ? lo_l : t_lo[tp(i)], id = last ? iden_l : t_id[tp(i)];
      v = (x[k] - l * v) * id;
      x[k] = v;
    }
  }
  // back substitution m_i = d'_i - cp_i m_{i+1}
  A = lift<R>(1.0);
  v = zero;
#pragma unroll
  for (int k = kSeg - 1; k >= 0; --k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R c = (i == n - 1) ? zero : t_cp[tp(i)];
      v = x[k] - c * v;
      A = -c * A;
    }
  }
  v = segment_carry_in<R>(A, v, true);
#pragma unroll
  for (int k = kSeg - 1; k >= 0; --k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R c = (i == n - 1) ? zero : t_cp[tp(i)];
      v = x[k] - c * v;
      x[k] = v;
    }
  }
  // m_1, m_2, m_{n-2}, m_{n-1} for the eliminated end values
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt) {
      if (i == 1) smem4[0] = x[k];
      if (i == 2) smem4[1] = x[k];
      if (i == n - 2) smem4[2] = x[k];
      if (i == n - 1) smem4[3] = x[k];
    }
  }
  __syncwarp();
  const R h0 = t_h[tp(0)], h1 = t_h[tp(1)], ha = t_h[tp(n - 2)], hb = t_h[tp(n - 1)];
  const R m0 = ((h0 + h1) * smem4[0] - h0 * smem4[1]) / h1;
  const R mn = ((ha + hb) * smem4[3] - hb * smem4[2]) / ha;
  const R next_first = warp_shfl_down(x[0], 1);  // m at row i0 + cnt (when it is a row)
  const R sixth = lift<R>(1.0 / 6.0), half = lift<R>(0.5), two = lift<R>(2.0);
  FF yc = y[fit_pad(i0)];
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt) {
      const R mi = (i == 0) ? m0 : x[k];
      R mj;
      if (i + 1 == n) mj = mn;
      else if (k + 1 < cnt) mj = x[(k + 1) < kSeg ? k + 1 : k];
      else mj = next_first;
      const FF yn = y[fit_pad(i + 1)];
      const FF slf = (yn - yc) * t_gih[tp(i)];
      const R corr = t_h[tp(i)] * (two * mi + mj) * sixth;
      const R cc = half * mi;
      const R dc = (mj - mi) * t_ih[tp(i)] * sixth;
      if constexpr (std::is_same<R, FF>::value) {
        FF* o = M.cphi + ((size_t)sd * M.J + i) * 4;
        o[0] = yc;
        o[1] = slf - corr;
        o[2] = cc;
        o[3] = dc;
      } else {
        // b = slope - h (2 m_i + m_j) / 6 from the float-float slope: FP32 head and tail
        const FF bf = ff_addf(slf, -corr);
        M.cg[((size_t)sd * M.J + i) * 8 + (q - 1)] = make_float4(yc.hi, bf.hi, cc, dc);
        reinterpret_cast<float*>(M.cg + ((size_t)sd * M.J + i) * 8 + 6)[q - 1] = yc.lo;
        M.cgb[((size_t)sd * M.J + i) * 6 + (q - 1)] = bf.lo;
      }
      yc = yn;
    }
  }
}

// kFitWarps systems per block.  R = FF: the phase systems (one per sample and
// detector, q = 0); R = float: the six transfer systems (q = 1..6).
template <int kSeg, class R>
__global__ void __launch_bounds__(kFitWarps * 32, 3) k_spline_fit(MixedDev M, int64_t n_sys) {
  extern __shared__ __align__(16) unsigned char fit_smem[];
  constexpr bool kPhase = std::is_same<R, FF>::value;
  constexpr bool kStage = kSeg == 32;
  const int rows = fit_rows(M.J);
  const R* src = kPhase ? reinterpret_cast<const R*>(M.gff) : reinterpret_cast<const R*>(M.gf);
  R* t_h = reinterpret_cast<R*>(fit_smem);
  R* t_ih = t_h + rows;
  R* t_lo = t_ih + rows;
  R* t_id = t_lo + rows;
  R* t_cp = t_id + rows;
  FF* t_gih = kPhase ? reinterpret_cast<FF*>(t_ih) : reinterpret_cast<FF*>(t_cp + rows);
  const size_t tables = kStage ? 5 * (size_t)rows * sizeof(R) + (kPhase ? 0 : (size_t)rows * sizeof(FF)) : 0;
  unsigned char* wbase = fit_smem + ((tables + 15) & ~(size_t)15);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  FF* ys = reinterpret_cast<FF*>(wbase + (size_t)warp * (rows * sizeof(FF) + 4 * sizeof(FF)));
  R* sm4 = reinterpret_cast<R*>(ys + rows);
  if (!kStage) {
    t_h = const_cast<R*>(src + (size_t)kGfH * M.J);
    t_ih = const_cast<R*>(src + (size_t)kGfInvH * M.J);
    t_lo = const_cast<R*>(src + (size_t)kGfLo * M.J);
    t_id = const_cast<R*>(src + (size_t)kGfInvDen * M.J);
    t_cp = const_cast<R*>(src + (size_t)kGfCp * M.J);
    t_gih = const_cast<FF*>(M.gff + (size_t)kGfInvH * M.J);
  }
  // shared grid tables (coalesced)
  if (kStage) {
    const int which[5] = {kGfH, kGfInvH, kGfLo, kGfInvDen, kGfCp};
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      R* dst = t_h + (size_t)t * rows;
      const R* sp = src + (size_t)which[t] * M.J;
      for (int i = threadIdx.x; i < M.J; i += blockDim.x) dst[fit_pad(i)] = sp[i];
    }
    if (!kPhase) {
      const FF* sp = M.gff + (size_t)kGfInvH * M.J;
      for (int i = threadIdx.x; i < M.J; i += blockDim.x) t_gih[fit_pad(i)] = sp[i];
    }
  }
  __syncthreads();
  const int64_t sys = (int64_t)blockIdx.x * kFitWarps + warp;
  if (sys >= n_sys) return;
  const int64_t sd = kPhase ? sys : sys / 6;
  const int q = kPhase ? 0 : 1 + (int)(sys % 6);
  const int n = M.nsp[sd / M.n_det];
  if (n < 3) return;
  const FF* yq = M.yv + ((size_t)sd * kNodeQ + q) * M.J;
  for (int i = lane; i <= n; i += 32) ys[fit_pad(i)] = yq[i];
  __syncwarp();
  spline_fit_staged<kSeg, R, kStage>(M, sd, q, n, t_h, t_ih, t_lo, t_id, t_cp, t_gih, ys, sm4);
}

// Transpose of the fit with the same lane segments.  mom(i, p) gives the
// interval moments, the tables are indexed through tp (padded rows when they
// were staged in shared memory).
template <int kSeg, class R, class MomAt, class TabIdx>
__device__ __forceinline__ void spline_adjoint_seg(const MixedDev& M, int64_t sd, int q, int n, int seg, double wscale,
                                                   const R* __restrict__ fh, const R* __restrict__ fih,
                                                   const R* __restrict__ flo, const R* __restrict__ fup,
                                                   const R* __restrict__ fid, MomAt mom, TabIdx tp) {
  const int lane = threadIdx.x & 31;
  float* __restrict__ yb = M.ybar + (size_t)sd * M.J * kNodeQ + q;
  const int i0 = min(n, lane * seg), cnt = min(n, i0 + seg) - i0;
  const R ws = (R)wscale;
  auto mm = [&](int i, int p) { return ws * (R)mom(i, p); };
  auto mbar_left = [&](int i) {
    return -fh[tp(i)] * mm(i, 1) * R(1.0 / 3.0) + R(0.5) * mm(i, 2) - mm(i, 3) * fih[tp(i)] * R(1.0 / 6.0);
  };
  auto mbar_right = [&](int i) { return -fh[tp(i)] * mm(i, 1) * R(1.0 / 6.0) + mm(i, 3) * fih[tp(i)] * R(1.0 / 6.0); };
  const R mb0 = mbar_left(0), mbn = mbar_right(n - 1);
  const R h0 = fh[tp(0)], h1 = fh[tp(1)], ha = fh[tp(n - 2)], hb = fh[tp(n - 1)];
  double lo_d, di_d, up_d;
  nak_row(M.node_f, n, n - 1, lo_d, di_d, up_d);
  const R lo_l = (R)lo_d, iden_l = (R)(1.0 / (di_d - lo_d * M.gcp[n - 2]));
  // right-hand sides (coefficient adjoints -> mbar, end eliminations), in FP64
  R x[kSeg];
  {
    R right_prev = (i0 >= 1) ? mbar_right(i0 - 1) : R(0);
#pragma unroll
    for (int k = 0; k < kSeg; ++k) {
      x[k] = R(0);
      const int i = i0 + k;
      if (k < cnt) {
        const R left = mbar_left(i);
        if (i >= 1) {
          R w = right_prev + left;
          if (i == 1) w += mb0 * (h0 + h1) / h1;
          if (i == 2) w -= mb0 * h0 / h1;
          if (i == n - 1) w += mbn * (ha + hb) / ha;
          if (i == n - 2) w -= mbn * hb / ha;
          x[k] = w;
        }
        right_prev = mbar_right(i);
      }
    }
  }
  // U^T z = mbar
  R A = R(1), v = R(0);
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R sub = (i > 1) ? fup[tp(i - 1)] : R(0), id = (i == n - 1) ? iden_l : fid[tp(i)];
      v = (x[k] - sub * v) * id;
      A = -sub * id * A;
    }
  }
  v = segment_carry_in<R>(A, v, false);
#pragma unroll
  for (int k = 0; k < kSeg; ++k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R sub = (i > 1) ? fup[tp(i - 1)] : R(0), id = (i == n - 1) ? iden_l : fid[tp(i)];
      v = (x[k] - sub * v) * id;
      x[k] = v;
    }
  }
  // L^T rbar = z
  A = R(1);
  v = R(0);
#pragma unroll
  for (int k = kSeg - 1; k >= 0; --k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R c = (i == n - 1) ? R(0) : ((i + 1 == n - 1) ? lo_l : flo[tp(i + 1)]) * fid[tp(i)];
      v = x[k] - c * v;
      A = -c * A;
    }
  }
  v = segment_carry_in<R>(A, v, true);
  R last = R(0);  // rbar of the segment's last row
#pragma unroll
  for (int k = kSeg - 1; k >= 0; --k) {
    const int i = i0 + k;
    if (k < cnt && i >= 1) {
      const R c = (i == n - 1) ? R(0) : ((i + 1 == n - 1) ? lo_l : flo[tp(i + 1)]) * fid[tp(i)];
      v = x[k] - c * v;
      x[k] = v;
      if (k == cnt - 1) last = v;
    }
  }
  // node adjoints ybar_i = Dbar_{i-1}/h_{i-1} + wscale mm0_i - Dbar_i/h_i,
  // Dbar_i = wscale mm1_i + 6 (rbar_i - rbar_{i+1}); rbar_0 = rbar_n = 0
  const R prev_last = __shfl_up_sync(0xffffffffu, last, 1);
  const R next_first = __shfl_down_sync(0xffffffffu, x[0], 1);
  double gd = 0.0;
  if (cnt > 0) {
    R dprev = R(0);
    if (i0 > 0) {
      const R r_prev = (i0 - 1 >= 1) ? prev_last : R(0);
      dprev = (mm(i0 - 1, 1) + R(6) * (r_prev - x[0])) * fih[tp(i0 - 1)];
    }
#pragma unroll
    for (int k = 0; k < kSeg; ++k) {
      const int i = i0 + k;
      if (k < cnt) {
        const R rc = (i >= 1) ? x[k] : R(0);
        R rn;
        if (i + 1 >= n) rn = R(0);
        else if (k + 1 < cnt) rn = x[(k + 1) < kSeg ? k + 1 : k];
        else rn = next_first;
        const R Db = mm(i, 1) + R(6) * (rc - rn);
        yb[i * kNodeQ] = (float)(dprev + mm(i, 0) - Db * fih[tp(i)]);
        dprev = Db * fih[tp(i)];
        if (q == 0) gd += 2.0 * kPi * (M.node_f[i] * (double)mom(i, 0) +
                                       (double)mom(i, 1));
      }
    }
    if (i0 + cnt == n) yb[n * kNodeQ] = (float)dprev;
  }
  for (int i = n + 1 + lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
  if (q == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gd += __shfl_xor_sync(0xffffffffu, gd, o);
    if (lane == 0) M.gdir[sd] = wscale * gd;
  }
}

// Register-segment adjoint, one system per warp, moments and tables read
// lane-strided from global memory (grids of more than 32 x 32 intervals).
template <int kSeg>
__global__ void __launch_bounds__(32) k_spline_adjoint(MixedDev M, double wscale) {
  const int q = (int)(blockIdx.x % kNodeQ), lane = threadIdx.x & 31;
  const int64_t sd = blockIdx.x / kNodeQ;
  const int n = M.nsp[sd / M.n_det];
  if (n < 3) {
    float* yb = M.ybar + (size_t)sd * M.J * kNodeQ + q;
    for (int i = lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
    if (q == 0 && lane == 0) M.gdir[sd] = 0.0;
    return;
  }
  const float* mom = M.mom + (size_t)sd * M.J * kNodeQ * kMoments + (size_t)q * kMoments;
  auto mat = [mom](int i, int p) { return mom[(size_t)i * kNodeQ * kMoments + p]; };
  auto tp = [](int i) { return i; };
  if (q == 0)
    spline_adjoint_seg<kSeg, double>(M, sd, q, n, (n + 31) >> 5, wscale, spline_factor<double>(M, kGfH),
                                     spline_factor<double>(M, kGfInvH), spline_factor<double>(M, kGfLo),
                                     spline_factor<double>(M, kGfUp), spline_factor<double>(M, kGfInvDen), mat, tp);
  else
    spline_adjoint_seg<kSeg, float>(M, sd, q, n, (n + 31) >> 5, wscale, spline_factor<float>(M, kGfH),
                                    spline_factor<float>(M, kGfInvH), spline_factor<float>(M, kGfLo),
                                    spline_factor<float>(M, kGfUp), spline_factor<float>(M, kGfInvDen), mat, tp);
}

// Staged adjoint (32-row segments): kFitWarps systems per block; the block
// copies the grid tables (h, 1/h, lo, up, 1/den; FP64 for the phase systems,
// FP32 for the transfer ones) and each warp its system's four moments per
// interval to shared memory with coalesced loads.
template <class R>
__host__ __device__ __forceinline__ size_t adj_smem_bytes(int J) {
  const size_t rows = (size_t)fit_rows(J);
  return ((5 * rows * sizeof(R) + 15) & ~(size_t)15) + (size_t)kFitWarps * rows * sizeof(float4);
}

template <class R>
__global__ void __launch_bounds__(kFitWarps * 32) k_spline_adjoint_staged(MixedDev M, int64_t n_sys, double wscale) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  constexpr bool kPhase = std::is_same<R, double>::value;
  const int rows = fit_rows(M.J);
  R* tab = reinterpret_cast<R*>(adj_smem);
  const int which[5] = {kGfH, kGfInvH, kGfLo, kGfUp, kGfInvDen};
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const R* src = spline_factor<R>(M, which[t]);
    for (int i = threadIdx.x; i < M.J; i += blockDim.x) tab[(size_t)t * rows + fit_pad(i)] = src[i];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sys = (int64_t)blockIdx.x * kFitWarps + warp;
  if (sys >= n_sys) return;
  const int64_t sd = kPhase ? sys : sys / 6;
  const int q = kPhase ? 0 : 1 + (int)(sys % 6);
  const int n = M.nsp[sd / M.n_det];
  if (n < 3) {
    float* yb = M.ybar + (size_t)sd * M.J * kNodeQ + q;
    for (int i = lane; i < M.J; i += 32) yb[i * kNodeQ] = 0.0f;
    if (q == 0 && lane == 0) M.gdir[sd] = 0.0;
    return;
  }
  float4* ms = reinterpret_cast<float4*>(adj_smem + ((5 * (size_t)rows * sizeof(R) + 15) & ~(size_t)15)) +
               (size_t)warp * rows;
  const float* mom = M.mom + (size_t)sd * M.J * kNodeQ * kMoments + (size_t)q * kMoments;
  for (int i = lane; i < n; i += 32)
    ms[fit_pad(i)] = *reinterpret_cast<const float4*>(mom + (size_t)i * kNodeQ * kMoments);
  __syncwarp();
  auto mat = [ms](int i, int p) {
    const float4 v = ms[fit_pad(i)];
    return p == 0 ? v.x : (p == 1 ? v.y : (p == 2 ? v.z : v.w));
  };
  spline_adjoint_seg<32, R>(M, sd, q, n, 32, wscale, tab, tab + rows, tab + 2 * rows, tab + 3 * rows, tab + 4 * rows,
                            mat, [](int i) { return fit_pad(i); });
}

// ------------------------------------------------------------------ exact bins
// Error model that decides which samples are re-evaluated over their dense
// range (the bar is |dlnL| <= 1e-2 against the FP64 evaluation).  The dense
// stage adds back the splines' midpoint error (k_bump), so what is left is
// (a) the FP32 rounding of the model in the cross term, a sum of independent
// per-bin errors whose spread is about 2.2e-7 sqrt(sum |d|^2 |h|^2 w^2)
// (times 2 df, in lnL), modelled as kCrossRel = 4e-7 times that root sum (for
// several modes the root sum takes sum (|d|^2 + |h|^2) |h|^2 w^2, which also
// bounds the modes' cross terms h_k conj(h_l) w); and (b) the part of the
// splines' error that the midpoint bump does not capture, modelled as
// kSplineRel of the intervals' absolute midpoint estimates of sum |h|^2 w.  A
// sample is refined when the two exceed kRefineTarget: the unrefined ones
// then have a rounding spread below 2.2e-3, which puts the 1e-2 bar at 4.5 of
// those spreads.  A refined sample whose spline part alone stays within the
// target is re-evaluated in float-float from the same splines (its rounding
// drops out, k_dense_ff); one above it, exactly (k_exact<3>).
constexpr double kRefineTarget = 4e-3;
constexpr double kCrossRel = 4e-7;
constexpr double kSplineRel = 0.01;
// Six-mode plans: the summed modes of heavy templates (dense range within the
// lowest eighth of the grid) carry a coherent model error of up to about
// 2e-9 of sum |h|^2 w in their merger-ringdown band, which the midpoint
// estimate does not see (measured on the three-detector network).  Those
// whose power puts that above the 1e-2 bar are re-evaluated exactly: few
// samples, and few bins each.
constexpr double kModelRelHM = 2e-9;
constexpr double kBar = 1e-2;

// one thread per sample, after the dense stage (its rounding sums) and k_hd
__global__ void k_refine_select(PlanDev P, MixedDev M, const SampleBlock<double>* __restrict__ blocks, int64_t B) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  int kind = kRefineNone;
  if (blocks[s].status == kSampleOk) {
    double sq = 0.0, eha = 0.0, hh = 0.0;
    for (int k = 0; k < M.nblk_dense; ++k) sq += M.part[((size_t)s * M.nblk_dense + k) * kPartW + 3];
    for (int k = 0; k < M.n_modes; ++k)
      for (int d = 0; d < M.n_det; ++d) {
        const double* hv = M.hd + (((size_t)s * M.n_modes + k) * M.n_det + d) * kHdOut;
        eha += hv[4];
        hh += hv[0];
      }
    const double er = 2.0 * P.df * kCrossRel * sqrt(fmax(sq, 0.0));
    const double es = 2.0 * P.df * kSplineRel * eha;
    const bool heavy = M.n_modes > 1 && blocks[s].kcut * 8 <= P.nbins;
    const bool loud = heavy && 2.0 * P.df * kModelRelHM * fabs(hh) > kBar;
    if (M.refine_all || er + es > kRefineTarget || loud)
      kind = (es > kRefineTarget || loud) ? kRefineExact : kRefineFF;
  }
  M.rkind[s] = kind;
}

// Bins [0, xbind[s][d]) of each detector evaluated directly (FP64 model and residual against the
// FP64 data).  kMode 0: lnL partials (T = double); 1: gradient partials
// (T = GradScalar, FP64 values with FP32 tangents); 2: write the model;
// 3: lnL partials of bins [xbind[s][d], kcut) of the samples that
// k_refine_select sends to the exact re-evaluation of their dense range
// (without the T-channel zero windows); 4: lnL partials of the window bins
// in [xbind[s][d], kcut) (their gradient: k_zero_grad).
// grid (xblocks, rblocks or zblocks, B); threads stride over the bins.  The
// value passes are held to 168 registers (3 blocks per SM instead of 2: the
// bench step 1.5% faster).
template <int kMode, class T>
__global__ void __launch_bounds__(kExactThreads, kMode == 1 ? 1 : 3) k_exact(PlanDev P, MixedDev M, GenArg G,
                                                         const SampleBlock<T>* __restrict__ blocks,
                                                         double2* __restrict__ model) {
  constexpr bool kGradPass = kMode == 1;
  constexpr int NV = kGradPass ? 11 : 1;
  constexpr bool kFF = !kGradPass;  // value passes: float-float values
  constexpr bool kRefine = kMode == 3;
  constexpr bool kZero = kMode == 4;  // the T-channel zero windows
  // value passes: a float-float copy of the block; gradient passes: the split
  // float-float block (mass/spin and response tangents)
  using SBF = std::conditional_t<kGradPass, ExactGradBlock, SampleBlock<FF>>;
  __shared__ SampleBlock<T> sb;
  __shared__ SBF sbf;
  __shared__ double red[kExactThreads / 32][NV];
  __shared__ PhenomHMCoef<double> hmd;  // multi-mode plans (value passes)
  __shared__ PhenomHMCoef<FF> hmf;
  const int s = blockIdx.y;
  const int nm = M.n_modes;
  const int xb = M.xbin[(size_t)s * nm];
  if (!kRefine && !kZero && xb == 0) return;  // uniform per block; the finalizers skip such samples
  if (kRefine && (blocks[s].status != kSampleOk || M.rkind[s] != kRefineExact)) return;
  load_block(blocks, s, sb);
  if (kFF && M.hm) load_hm(M.hm, s, hmd);
  __syncthreads();
  if constexpr (kFF) {
    narrow_block_ff(sb, sbf);
    if (M.hm) narrow_hm_ff(hmd, hmf);
  } else {
    narrow_exact_grad(sb, sbf);
  }
  __syncthreads();
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  const double inv_scale = 1.0 / M.scale;
  if (sb.status == kSampleOk) {
    for (int d = 0; d < M.n_det; ++d) {
      const int xbd = M.xbind[(size_t)s * nm * M.n_det + d];
      const int i0 = kRefine ? xbd : 0, i1 = kRefine ? (int)sb.kcut : xbd;
      const int n_it = kZero ? M.nzb[d] : i1 - i0;
      for (int it = blockIdx.x * kExactThreads + threadIdx.x; it < n_it; it += gridDim.x * kExactThreads) {
        int i = i0 + it;
        if constexpr (kZero) {
          i = M.zbin[(size_t)d * kZeroMax + it];
          if (i < xbd || i >= (int)sb.kcut) continue;  // below: the exact low bins take it
        }
        if constexpr (kRefine) {
          if (in_zero_window(M, d, i)) continue;  // the window kernel takes it
        }
        if constexpr (kFF) {
          const FF f = ff_mulf(M.fstep_ff, (float)(P.k0 + i));  // k0 + i < 2^24: exact in FP32
          const TdiFactor& tdb = P.tdi[(size_t)d * P.nbins + i];
          // the modes' channels in float-float, summed
          FF hsr[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
          FF hsi[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
#pragma unroll 1
          for (int k = 0; k < nm; ++k) {
            FF y[kNodeQ];
            bool live = true;
            node_eval_mode<true, FF>(M.orbit_ff[d], M.scale_ff, sbf, M.hm ? &hmf : nullptr, k,
                                     cx(ff_from(tdb.dre), ff_from(tdb.dim)), cx(ff_from(tdb.pre), ff_from(tdb.pim)),
                                     f, y, &live);
            if (!live) continue;  // the mode above its mapped Mf = 0.2
            // phase reduced modulo 2 pi in FP64, then its sine and cosine in FF
            const double phd = ff_to(y[0] + (2.0 * kPi * f) * sbf.tc);
            FF sn, cs;
            dsincos(ff_from(phd - (2.0 * kPi) * rint(phd * (1.0 / (2.0 * kPi)))), &sn, &cs);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
              hsr[ch] = hsr[ch] + (y[1 + 2 * ch] * cs + y[2 + 2 * ch] * sn);
              hsi[ch] = hsi[ch] + (y[2 + 2 * ch] * cs - y[1 + 2 * ch] * sn);
            }
          }
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            const double hr = ff_to(hsr[ch]) * inv_scale;
            const double hi = ff_to(hsi[ch]) * inv_scale;
            const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
            if constexpr (kMode == 2) {
              model[off] = make_double2(hr, hi);
            } else {
              const double w = P.w[off];
              const double2 dv = P.data[off];
              const double rr = dv.x - hr, ri = dv.y - hi;
              acc[0] += w * (rr * rr + ri * ri);
            }
          }
          continue;
        }
        if constexpr (kGradPass) {
          const double f = (double)(P.k0 + i) * P.f_step;
          const TdiFactor& tdb = P.tdi[(size_t)d * P.nbins + i];
          // PhenomD with the mass/spin tangents
          EM amp, psi, tf;
          phenomd_eval<EM>(sbf.wf, sbf.wf.Msec * f, amp, psi, tf);
          amp = amp * M.scale;
          // response per unit amplitude with the T and sky/orientation tangents
          Cx<ER> Y[3];
          ER kx0;
          {
            ER T = lift<ER>(0.0);
            T.v = tf.v + sbf.tc;
            T.d[0] = 1.0f;
            const ER zero = lift<ER>(0.0);
            Cx<ER> L[6];
            single_links_impl<true, ER>(P.orbit[d], f, cx(sbf.pfac, zero), cx(zero, -sbf.cfac), T, sbf.pol, L, &kx0);
            tdi_channels<ER>(cx(tdb.dre, tdb.dim), cx(tdb.pre, tdb.pim), 1, L, Y);
          }
          // phase Psi + 2 pi f (k.x0 + t_c), whole turns removed in FP64 (it reaches 1e6 rad)
          FF sn, cs;
          {
            const double phd = ff_to(psi.v + (2.0 * kPi * f) * (kx0.v + sbf.tc));
            dsincos(ff_from(phd - (2.0 * kPi) * rint(phd * (1.0 / (2.0 * kPi)))), &sn, &cs);
          }
          const float csf = cs.hi, snf = sn.hi, ampf = amp.v.hi;
          // per channel: E = conj(d - h) e^{-i ph} / scale, and with X = Y or a
          // tangent of Y, Re(E X) and Im(E Y) (the phase derivative's factor)
          float A0 = 0.0f, A1 = 0.0f, BT = 0.0f, Br[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            const FF yr = amp.v * Y[ch].re.v, yi = amp.v * Y[ch].im.v;
            const double hr = ff_to(yr * cs + yi * sn) * inv_scale;
            const double hi = ff_to(yi * cs - yr * sn) * inv_scale;
            const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
            const double w = P.w[off];
            const double2 dv = P.data[off];
            const double rr = dv.x - hr, ri = dv.y - hi;
            acc[4] += 2.0 * w * (rr * hr + ri * hi);  // dh/dlnD_L = -h
            acc[9] += 4.0 * w * (rr * hi - ri * hr);  // dh/dphi_c = 2 i h
            // -2 w E in FP64: w / scale alone can exceed the FP32 range (w = 1/S), the product is O(1)
            const double m2w = -2.0 * w * inv_scale;
            const double csd = (double)csf, snd = (double)snf;
            const float er = (float)(m2w * (rr * csd - ri * snd)), ei = (float)(-m2w * (rr * snd + ri * csd));
            const ER& Yr = Y[ch].re;
            const ER& Yi = Y[ch].im;
            A0 = fmaf(er, Yr.v.hi, fmaf(-ei, Yi.v.hi, A0));
            A1 = fmaf(er, Yi.v.hi, fmaf(ei, Yr.v.hi, A1));
            BT = fmaf(er, Yr.d[0], fmaf(-ei, Yi.d[0], BT));
#pragma unroll
            for (int k = 0; k < 4; ++k) Br[k] = fmaf(er, Yr.d[1 + k], fmaf(-ei, Yi.d[1 + k], Br[k]));
          }
          A1 *= ampf;
          BT *= ampf;
          const float tpf = (float)(2.0 * kPi * f);
          float g[kMixNT];
#pragma unroll
          for (int k = 0; k < 4; ++k) g[k] = A0 * amp.d[k] + BT * tf.d[k] + A1 * (psi.d[k] + tpf * kx0.d[0] * tf.d[k]);
          g[4] = ampf * Br[3] + A1 * tpf * kx0.d[4];  // cos iota
          g[5] = ampf * Br[0] + A1 * tpf * kx0.d[1];  // lambda
          g[6] = ampf * Br[1] + A1 * tpf * kx0.d[2];  // sin beta
          g[7] = ampf * Br[2] + A1 * tpf * kx0.d[3];  // psi
          g[8] = BT + A1 * tpf * (kx0.d[0] + 1.0f);   // t_c
#pragma unroll
          for (int k = 0; k < kMixNT; ++k) acc[kSlotParam[k]] += (double)g[k];
        }
      }
    }
  }
  if (kMode == 2) return;
  const int wid = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (l == 0) red[wid][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < kExactThreads / 32; ++w) x += red[w][threadIdx.x];
    if (kMode == 0)
      M.xpart[(size_t)s * gridDim.x + blockIdx.x] = x;
    else if (kMode == 3)
      M.rpart[(size_t)s * gridDim.x + blockIdx.x] = x;
    else if (kMode == 4)
      M.zpart[(size_t)s * gridDim.x + blockIdx.x] = x;
    else
      M.xgpart[((size_t)s * gridDim.x + blockIdx.x) * 11 + threadIdx.x] = x;
  }
}

// Gradient of the T-channel zero windows (one-mode plans): d/dtheta of
// sum_c |d - h|^2 w over each window bin in [xbind, kcut) of each detector,
// with FP64 dual numbers over the 11 parameters (near T's zero its transfer
// is a cancellation of the links that FP32 tangents cannot resolve, and the
// weight 1/S_T amplifies what they miss).  grid (zblocks, B).
using ZScalar = Dual<11>;
__device__ __forceinline__ ZScalar zero_bin_residual(const PlanDev& P, const SampleBlock<ZScalar>& b, int d,
                                                     int64_t i) {
  using T = ZScalar;
  const double f = (double)(P.k0 + i) * P.f_step;
  T amp, psi, tf;
  phenomd_eval<T>(b.wf, b.wf.Msec * f, amp, psi, tf);
  T sn, cs;
  dsincos(psi, &sn, &cs);
  const T ap = b.wf.pfac * amp, ac = b.wf.cfac * amp;
  Cx<T> hp = cx(ap * cs, -(ap * sn));
  Cx<T> hc = cx(-(ac * sn), -(ac * cs));
  Cx<T> ts;
  dsincos((-2.0 * kPi * f) * b.tc, &ts.im, &ts.re);
  hp = cmul(hp, ts);
  hc = cmul(hc, ts);
  Cx<T> L[6], C[3];
  single_links<T>(P.orbit[d], f, hp, hc, tf + b.tc, b.pol, L);
  const TdiFactor dp = P.tdi[(size_t)d * P.nbins + i];
  tdi_channels<T>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), 1, L, C);
  T sum = lift<T>(0.0);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    if (!((P.chan_mask >> ch) & 1)) continue;
    const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
    const double2 dv = P.data[off];
    const T rr = dv.x - C[ch].re, ri = dv.y - C[ch].im;
    sum = sum + (rr * rr + ri * ri) * P.w[off];
  }
  return sum;
}

__global__ void __launch_bounds__(kExactThreads) k_zero_grad(PlanDev P, MixedDev M,
                                                             const SampleBlock<ZScalar>* __restrict__ blocks) {
  __shared__ SampleBlock<ZScalar> sb;
  __shared__ double red[kExactThreads / 32][11];
  const int s = blockIdx.y;
  {
    const int n8 = sizeof(SampleBlock<ZScalar>) / 8;
    const double* src = reinterpret_cast<const double*>(&blocks[s]);
    double* dst = reinterpret_cast<double*>(&sb);
    for (int j = threadIdx.x; j < n8; j += blockDim.x) dst[j] = src[j];
  }
  __syncthreads();
  double acc[11];
#pragma unroll
  for (int k = 0; k < 11; ++k) acc[k] = 0.0;
  if (sb.status == kSampleOk) {
    for (int d = 0; d < M.n_det; ++d) {
      const int xbd = M.xbind[(size_t)s * M.n_det + d];
      for (int it = blockIdx.x * kExactThreads + threadIdx.x; it < M.nzb[d]; it += gridDim.x * kExactThreads) {
        const int i = M.zbin[(size_t)d * kZeroMax + it];
        if (i < xbd || i >= (int)sb.kcut) continue;  // below: the exact low bins take it
        const ZScalar r = zero_bin_residual(P, sb, d, i);
#pragma unroll
        for (int k = 0; k < 11; ++k) acc[k] += r.d[k];
      }
    }
  }
  const int wid = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 11; ++k) {
    double x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (l == 0) red[wid][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < 11) {
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < kExactThreads / 32; ++w) x += red[w][threadIdx.x];
    M.zgpart[((size_t)s * gridDim.x + blockIdx.x) * 11 + threadIdx.x] = x;
  }
}

// ------------------------------------------------------------------ dense stage
// 2 pi split into a 12-bit head and two tails for exact FP32 reduction of
// exactly-representable arguments up to ~2^11 turns.
constexpr float kTwoPiHi = 6.28125f;                // 8 significant bits: k * hi exact for |k| < 2^16
constexpr float kTwoPiMid = 0.0019353071693331003f;   // float(2 pi - hi)
constexpr float kTwoPiLo = 1.0253131677018246e-11f;   // float(2 pi - hi - mid)
constexpr float kInvTwoPi = 0.159154943091895336f;

constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23: (y + M) - M rounds |y| < 2^22 to an integer

__device__ __forceinline__ float reduce_exact(float x) {
  const float k = fmaf(x, kInvTwoPi, kRoundMagic) - kRoundMagic;
  float r = fmaf(-k, kTwoPiHi, x);
  r = fmaf(-k, kTwoPiMid, r);
  r = fmaf(-k, kTwoPiLo, r);
  return r;
}

// The same reduction with its rounding kept: x - 2 pi k = r + *e to about
// 2^-46 of |r| (the first subtraction is exact; the errors of the two
// rounded ones are recovered with FMAs, r0 - r1 being exact).
__device__ __forceinline__ float reduce_exact_ff(float x, float* e) {
  const float k = fmaf(x, kInvTwoPi, kRoundMagic) - kRoundMagic;
  const float r0 = fmaf(-k, kTwoPiHi, x);
  const float r1 = fmaf(-k, kTwoPiMid, r0);
  const float e1 = fmaf(-k, kTwoPiMid, r0 - r1);
  const float r2 = fmaf(-k, kTwoPiLo, r1);
  const float e2 = fmaf(-k, kTwoPiLo, r1 - r2);
  *e = e1 + e2;
  return r2;
}

// sin and cos of |x| < 2^21 in FP32 FMA arithmetic only: x = k pi/2 + r with
// k the nearest integer (magic-number rounding, k read from the float's bits)
// and pi/2 in three parts (k * hi exact for |k| < 2^15), then Taylor
// polynomials on |r| <= pi/4 (truncation below 2e-9) and the quadrant swap.
constexpr float kTwoOverPi = 0.6366197466850281f;
constexpr float kPiO2Hi = 1.5703125f;
constexpr float kPiO2Mid = 0.0004838267923332751f;
constexpr float kPiO2Lo = 2.5632829192545614e-12f;

__device__ __forceinline__ void sincos_poly(float x, float* sp, float* cp) {
  const float kf = fmaf(x, kTwoOverPi, kRoundMagic);
  const int k = __float_as_int(kf) - __float_as_int(kRoundMagic);
  const float kr = kf - kRoundMagic;
  float r = fmaf(-kr, kPiO2Hi, x);
  r = fmaf(-kr, kPiO2Mid, r);
  r = fmaf(-kr, kPiO2Lo, r);
  const float r2 = r * r;
  float ps = fmaf(r2, 1.0f / 362880.0f, -1.0f / 5040.0f);
  ps = fmaf(ps, r2, 1.0f / 120.0f);
  ps = fmaf(ps, r2, -1.0f / 6.0f);
  const float sr = fmaf(ps * r2, r, r);
  float pc = fmaf(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
  pc = fmaf(pc, r2, -1.0f / 720.0f);
  pc = fmaf(pc, r2, 1.0f / 24.0f);
  pc = fmaf(pc, r2, -0.5f);
  const float cr = fmaf(pc, r2, 1.0f);
  float sv = (k & 1) ? cr : sr;
  float cv = (k & 1) ? sr : cr;
  if (k & 2) sv = -sv;
  if ((k + 1) & 2) cv = -cv;
  *sp = sv;
  *cp = cv;
}

// head of x truncated to `bits` significant bits (so that head * small integer is exact in FP32)
__device__ __forceinline__ float head_bits(double x, int bits) {
  const long long m = ~((1LL << (53 - bits)) - 1);
  return (float)__longlong_as_double(__double_as_longlong(x) & m);
}

__device__ __forceinline__ double wrap_2pi(double x) {
  return x - (2.0 * kPi) * rint(x * (1.0 / (2.0 * kPi)));
}

struct RunPhase {
  float x0;               // Msec f - Mf_peak at the run start (FP64, rounded once)
  float c0, s0;           // cos, sin of the anchored phase at the run start
  float p1h, p1l;         // per-bin increment (wrapped), head/tail
  float p2h, p2l;         // quadratic coefficient, head/tail
  float p3h, p3l;         // cubic coefficient, head/tail
  float qx0, qj;          // multi-mode plans: the straddled phase corner (Msec f - Mf_c at the run start, Jh)
};

// The phase of run c (first bin kb, interval j) of virtual sample s on
// detector d (sd = s * n_det + d) in float-float: the phase spline plus
// 2 pi f t_c at the run's first bin, wrapped (ph0), and the per-bin
// increment polynomial ph1 u + ph2 u^2 + ph3 u^3 (u = bins past the first;
// ph1 wrapped).  Past a multi-mode plan's phase corner its term is included;
// the corner that the run straddles is returned (qk, and Msec f - Mf_c at the
// run start and Jh in FP32) to be added per bin.
struct AnchorFF {
  FF ph0, ph1, ph2, ph3;
  FF fbf;         // frequency of the run's first bin
  float qx0, qj;  // the straddled corner (0 when none)
  int qk;         // its index, -1 when none
};
__device__ __forceinline__ AnchorFF run_anchor_ff(const PlanDev& P, const MixedDev& M, int s, size_t sd, int c,
                                                  int kb, int j) {
  AnchorFF A;
  const float4 sa = M.sff[2 * s];
  const FF tcf = ff_make(sa.x, sa.y), msf = ff_make(sa.z, sa.w);
  const FF* co = M.cphi + (sd * M.J + j) * 4;
  const FF a = co[0], b = co[1], cc = co[2], dd = co[3];
  const float2 nfj = M.node_ff[j];
  const FF fbf = ff_mulf(M.fstep_ff, (float)(P.k0 + kb));  // k0 + kb < 2^24: exact in FP32
  const FF t = fbf - ff_make(nfj.x, nfj.y);
  const FF ddt = dd * t;
  FF S0 = a + t * (b + t * (cc + ddt));
  FF S1 = b + t * (ff_mulf(cc, 2.0f) + ff_mulf(ddt, 3.0f));
  FF S2 = cc + ff_mulf(ddt, 3.0f);
  const FF D = M.fstep_ff;
  A.qx0 = 0.0f;
  A.qj = 0.0f;
  A.qk = -1;
  if (M.pkink) {
    // the phase's corner terms Jh (Msec f - Mf_c)^2: value, slope and
    // curvature at the run start for runs past the corner
    const FF mfb = msf * fbf;
    const float last = (float)(M.ch_len[c] - 1) * (msf * D).hi;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float4 k4 = M.pkink[2 * s + q];
      const FF xq = mfb - ff_make(k4.x, k4.y), jq = ff_make(k4.z, k4.w);
      if (xq.hi >= 0.0f) {
        S0 = S0 + jq * (xq * xq);
        S1 = S1 + ff_mulf(jq * (xq * msf), 2.0f);
        S2 = S2 + jq * (msf * msf);
      } else if (xq.hi + last > 0.0f) {
        A.qx0 = xq.hi;
        A.qj = jq.hi;
        A.qk = q;
      }
    }
  }
  // anchored phase S0 + 2 pi f t_c.  f t_c reaches 1e6 cycles; its fraction is
  // (k0 + kb) frac(f_step t_c) mod 1, taken exactly in 64-bit integers and
  // read out as two 23-bit floats; the sum is wrapped in float-float (FP64
  // beyond the wide wrap's range).
  FF ph0;
  {
    const unsigned long long pr = (unsigned long long)(P.k0 + kb) * M.cfrac[s];
    const unsigned h23 = (unsigned)(pr >> 41), l23 = (unsigned)(pr >> 18) & 0x7FFFFFu;
    const float fh = (__uint_as_float(0x4B000000u | h23) - 8388608.0f) * 1.1920928955078125e-07f;   // / 2^23
    const float fl = (__uint_as_float(0x4B000000u | l23) - 8388608.0f) * 1.4210854715202004e-14f;  // / 2^46
    ph0 = S0 + ff_fast_two_sum(fh, fl) * (2.0 * kPi);
    if (fabsf(ph0.hi) < kWrapWideMax) {
      ph0 = ff_wrap_2pi_wide(ph0);
    } else {
      const double p = ff_to(ph0);
      ph0 = ff_from(p - (2.0 * kPi) * rint(p * (1.0 / (2.0 * kPi))));
    }
  }
  A.ph0 = ph0;
  A.ph1 = ff_wrap_2pi(D * (S1 + tcf * (2.0 * kPi)));
  A.ph2 = (D * D) * S2;
  A.ph3 = (D * D) * (D * dd);
  A.fbf = fbf;
  return A;
}

// Per-run phase anchors, one thread per (sample, detector, run) with a live,
// non-exact bin: the float-float anchor split into an FP32 head/tail phasor
// and exact-product FP32 heads (with tails) of the per-bin increment
// polynomial; and the peak-kink coordinate Msec f - Mf_peak at the run start.
__global__ void __launch_bounds__(128) k_run_anchors(PlanDev P, MixedDev M,
                                                      const SampleBlock<double>* __restrict__ blocks) {
  const int s = blockIdx.z, d = blockIdx.y;  // s: virtual sample (sample, mode)
  const int c = blockIdx.x * 128 + threadIdx.x;
  if (blocks[s / M.n_modes].status != kSampleOk || c >= M.nch[s]) return;
  const int kb = M.ch_begin[c];
  if (kb < M.xbind[(size_t)s * M.n_det + d]) return;
  const size_t sd = (size_t)s * M.n_det + d;
  const int j = M.ch_iv[c];
  const AnchorFF A = run_anchor_ff(P, M, s, sd, c, kb, j);
  const float4 sa = M.sff[2 * s], sbk = M.sff[2 * s + 1];
  const FF msf = ff_make(sa.z, sa.w), fpf = ff_make(sbk.x, sbk.y);
  const float x0 = (msf * A.fbf - fpf).hi;
  // anchor phasor: sincos of the float head, rotated by the (tiny) tail
  float s0f, c0f;
  sincos_poly(A.ph0.hi, &s0f, &c0f);
  const float l0 = A.ph0.lo;
  float p1l, p2l, p3l;
  const float p1h = ff_head(A.ph1, 12, &p1l), p2h = ff_head(A.ph2, 13, &p2l), p3h = ff_head(A.ph3, 8, &p3l);
  float4* o = M.runs + (sd * M.nchunks + c) * 3;
  o[0] = make_float4(x0, fmaf(-s0f, l0, c0f), fmaf(c0f, l0, s0f), p1h);
  o[1] = make_float4(p1l, p2h, p2l, p3h);
  o[2] = make_float4(p3l, A.qx0, A.qj, 0.0f);
}

// Warp-sum of the 28 per-lane interval moments through shared memory (rows
// padded to 33 floats: conflict-free), added to the interval's moments with
// one 28-lane atomic instruction.
constexpr int kMomPad = 33;
__device__ __forceinline__ void flush_moments(float mq[kNodeQ * kMoments], float (*sm)[kMomPad], float* dst,
                                              int lane) {
#pragma unroll
  for (int k = 0; k < kNodeQ * kMoments; ++k) {
    sm[k][lane] = mq[k];
    mq[k] = 0.0f;
  }
  __syncwarp();
  if (lane < kNodeQ * kMoments) {
    float x = 0.0f;
#pragma unroll 8
    for (int l = 0; l < 32; ++l) x += sm[lane][l];
    atomicAdd(dst + lane, x);
  }
  __syncwarp();
}

// Asynchronous 16-byte global -> shared copies (cp.async, completion by
// commit/wait groups: a thread's own copies, no spin loop).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(__cvta_generic_to_global(gmem))
               : "memory");
}
// the same through L1 (rows that the next runs of an interval read again)
__device__ __forceinline__ void cp_async16_l1(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(__cvta_generic_to_global(gmem))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// bring the line holding p into L1 (no register, no completion to wait for)
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];\n" ::"l"(__cvta_generic_to_global(p)));
}
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// One run's inputs in shared memory: the three packed rows of its (up to) 32
// bins, the interval's eight coefficient rows and the run's three anchor rows.
constexpr int kRunBuf = 3 * 32 + 8 + 3 + 2;  // packed bins, coefficient rows, anchor, midpoint corrections

// The splines' error at each interval's midpoint, against the exact model
// there, as the coefficients of a correction delta_q (4 t (h - t) / h^2)^2
// that the dense stage adds to each transfer quantity: the leading error term
// of cubic interpolation, f^(4)(xi) t^2 (h - t)^2 / 24, has this shape, so the
// corrected model also matches the exact one at the midpoints.  The phase
// spline's midpoint error dphi enters as a rotation of the exact transfer
// quantities, G e^{-i dphi}, since the model is G P e^{-i phase}.  One thread
// per (virtual sample, detector, interval).
__global__ void k_bump(MixedDev M, const SampleBlock<double>* __restrict__ blocks, int64_t B) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= B * M.n_modes * M.n_det * (int64_t)M.J) return;
  const int j = (int)(t % M.J);
  const int64_t sd = t / M.J;
  const int64_t v = sd / M.n_det;
  float4* out = M.cbump + (size_t)t * 2;
  if (blocks[v / M.n_modes].status != kSampleOk || M.nsp[v] < 3 || j >= M.nsp[v]) {
    out[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    out[1] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    return;
  }
  // float-float on the FP32 pipes: the midpoint errors are 1e-8..1e-6 of the
  // values, the phase error a small angle (its rotation to second order)
  const double h = M.gh[j];
  const FF tm = ff_from(0.5 * h);
  const FF* ym = M.ym + (size_t)sd * 7 * M.J + j;
  const FF* co = M.cphi + (size_t)t * 4;
  const FF phs = co[0] + tm * (co[1] + tm * (co[2] + tm * co[3]));
  const float dph = (ym[(size_t)6 * M.J] - phs).hi;
  const float sn = dph, cs = fmaf(-0.5f * dph, dph, 1.0f);
  const float4* cg = M.cg + (size_t)t * 8;
  const float* alo = reinterpret_cast<const float*>(cg + 6);
  const float* blo = M.cgb + (size_t)t * 6;
  const float tmf = tm.hi;
  float dl[6];
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    FF sp[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int q = 2 * ch + k;
      const float4 c4 = cg[q];
      // the value at the left node as float-float plus the (small) polynomial change
      sp[k] = ff_addf(ff_two_sum(c4.x, alo[q]), tmf * ((c4.y + blo[q]) + tmf * fmaf(tmf, c4.w, c4.z)));
    }
    const FF gr = ym[(size_t)(2 * ch) * M.J], gi = ym[(size_t)(2 * ch + 1) * M.J];
    dl[2 * ch] = (ff_addf(ff_mulf(gr, cs), gi.hi * sn) - sp[0]).hi;
    dl[2 * ch + 1] = (ff_addf(ff_mulf(gi, cs), -(gr.hi * sn)) - sp[1]).hi;
  }
  if (M.wspike[(size_t)(sd % M.n_det) * M.J + j]) {
#pragma unroll
    for (int q = 0; q < 6; ++q) dl[q] = 0.0f;
  }
  out[0] = make_float4(dl[0], dl[1], dl[2], dl[3]);
  out[1] = make_float4(dl[4], dl[5], (float)h, (float)(4.0 / (h * h)));
  if (M.n_modes > 1) {
    // the kink term C_q (X0 + Msec t)^2 of an interval past the kink point,
    // X0 = Msec f_j - Mf_kink >= 0, folded into its coefficients (FP64 sums,
    // value and slope kept as float-float)
    const SampleBlock<double>& b = blocks[v / M.n_modes];
    const float4 pk = M.sff[2 * v + 1];
    const double X0 = b.wf.Msec * M.node_f[j] - ff_to(ff_make(pk.x, pk.y));
    const int jk = (int)M.kinkF[(size_t)sd * 16 + 14];  // the interval holding the kink point
    if (jk >= 0 && j > jk) {
      const double* KC = M.kinkC + (size_t)sd * 6;
      float4* cgw = M.cg + (size_t)t * 8;
      float* alw = reinterpret_cast<float*>(cgw + 6);
      float* blw = M.cgb + (size_t)t * 6;
      const double ms = b.wf.Msec;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        float4 c4 = cgw[q];
        const double A = ((double)c4.x + (double)alw[q]) + KC[q] * X0 * X0;
        const double Bq = ((double)c4.y + (double)blw[q]) + 2.0 * KC[q] * X0 * ms;
        const double Cq = (double)c4.z + KC[q] * ms * ms;
        c4.x = (float)A;
        c4.y = (float)Bq;
        c4.z = (float)Cq;
        cgw[q] = c4;
        alw[q] = (float)(A - (double)c4.x);
        blw[q] = (float)(Bq - (double)c4.y);
      }
    }
  }
}

// kMode 0: lnL partials; 1: lnL partials + adjoint moments; 2: write the model
// h (unscaled, complex128 (n_det, 3, nbins)) to `model` (parity/debug path).
// kStage: the run inputs are copied one run ahead into shared memory (pays
// off when they stream from DRAM, and in the lnL pass; with L2-resident
// inputs the gradient pass is faster on plain loads).
// kNM: modes summed per bin before the residual (1, or kHMModes for
// IMRPhenomHM plans: lnL and model passes, plain loads).
// Every pass is held to 96 registers (5 blocks per SM, at a few spilled
// words): the gradient pass 2% faster than at 4 blocks, the staged lnL pass
// 6.5% (bench batch) and 17% (network, inputs from DRAM) faster than at 128
// registers, the six-mode pass 15% faster than at 4 blocks and 2 blocks.
template <int kMode, bool kStage, int kNM>
__global__ void __launch_bounds__(kMixThreads, 5) k_dense_mixed(PlanDev P, MixedDev M,
                                                             const SampleBlock<double>* __restrict__ blocks,
                                                             double2* __restrict__ model) {
  constexpr bool kGrad = kMode == 1;
  static_assert(kNM == 1 || (!kGrad && !kStage), "multi-mode dense stage: lnL and model passes, no staging");
  __shared__ double red[kMixThreads / 32][kPartW];
  // per warp, two run buffers: the next run's inputs are copied while this one is computed
  __shared__ __align__(16) float4 rbuf[kStage ? kMixThreads / 32 : 1][kStage ? 2 : 1][kStage ? kRunBuf : 1];
  __shared__ float msm[kGrad ? kMixThreads / 32 : 1][kGrad ? kNodeQ * kMoments : 1][kGrad ? kMomPad : 1];
  const int s = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int g = blockIdx.x * (kMixThreads / 32) + wid;  // run group
  int nc = M.nch[(size_t)s * kNM];  // runs with a live bin of any mode
#pragma unroll
  for (int k = 1; k < kNM; ++k) nc = max(nc, M.nch[(size_t)s * kNM + k]);
  const int64_t kcut = blocks[s].kcut;
  const int first = g * kChunkMax;
  float acc = 0.0f, comp = 0.0f;
  float dsh = 0.0f, dsl = 0.0f;  // float-float sum of the FP64 |d|^2/S of the weak-template bins
  float xacc = 0.0f, xcomp = 0.0f;  // compensated sum of the cross term -2 Re(d^* h) w
  float macc = 0.0f, mcomp = 0.0f;  // multi-mode plans: compensated sum of 2 Re sum_{k<l} h_k conj(h_l) w
  float sqa = 0.0f;  // rounding estimate: sum |d|^2 |h|^2 w^2 (several modes: (|d|^2 + |h|^2) |h|^2 w^2)
  if (blocks[s].status == kSampleOk && first < nc) {
    for (int d = 0; d < M.n_det; ++d) {
      const size_t sd = (size_t)s * kNM * M.n_det + d;  // (virtual sample of mode 0, detector)
      const int xb = M.xbind[sd];
      // ---- amplitude kink (float-float coefficients, read past the kink point only)
      const float kSlope = M.kinkF[sd * 16];  // Msec f_step, the same for every mode
      float km[12];
      bool kinked = false;
      if (kGrad) {
#pragma unroll
        for (int k = 0; k < 12; ++k) km[k] = 0.0f;
      }
      // ---- runs of the group, one bin per lane
      float mq[kNodeQ * kMoments];
      int cur_iv = -1;
      if (kGrad) {
#pragma unroll
        for (int k = 0; k < kNodeQ * kMoments; ++k) mq[k] = 0.0f;
      }
      const int last = min(nc, first + kChunkMax);
      // copy run c's inputs into buffer b (nothing for exact runs: runs never
      // straddle an interval boundary, and bins below xb are evaluated exactly)
      auto issue = [&](int c, int b) {
        if (c >= last) return;
        const int kb = M.ch_begin[c];
        if (kb < xb) return;
        float4* dst = &rbuf[wid][b][0];
        const int64_t i = (int64_t)kb + lane;
        if (lane < M.ch_len[c] && i < kcut) {
          const float4* pkd = M.pk + (size_t)d * 3 * P.nbins;
          cp_async16(dst + lane, pkd + i);
          cp_async16(dst + 32 + lane, pkd + P.nbins + i);
          cp_async16(dst + 64 + lane, pkd + 2 * P.nbins + i);
        }
        if (lane < 8)
          cp_async16_l1(dst + 96 + lane, M.cg + (sd * M.J + M.ch_iv[c]) * 8 + lane);
        else if (lane < 11)
          cp_async16(dst + 104 + (lane - 8), M.runs + (sd * M.nchunks + c) * 3 + (lane - 8));
        else if (lane < 13)
          cp_async16_l1(dst + 107 + (lane - 11), M.cbump + (sd * M.J + M.ch_iv[c]) * 2 + (lane - 11));
      };
      if (kStage) {
        issue(first, 0);
        cp_async_commit();
      }
      for (int c = first; c < last; ++c) {
        const int b = (c - first) & 1;
        if (kStage) {
          issue(c + 1, b ^ 1);
          cp_async_commit();
          cp_async_wait_one();  // run c's copies have landed
          __syncwarp();
        }
        const int j = M.ch_iv[c];
        const int kb = M.ch_begin[c];
        const int len = M.ch_len[c];
        if (kNM > 1 && c + 1 < last) {
          // touch the next run's inputs so that its loads hit L1: the L2 latency
          // of the six modes' rows at the top of each run stalls the loop (the
          // one-mode gradient pass ran 13% slower with these prefetches)
          const int kbn = M.ch_begin[c + 1];
          if (kbn >= xb) {
            const int64_t in = (int64_t)kbn + lane;
            if (lane < M.ch_len[c + 1] && in < kcut) {
              const float4* pkd = M.pk + (size_t)d * 3 * P.nbins;
              prefetch_l1(pkd + in);
              prefetch_l1(pkd + P.nbins + in);
              prefetch_l1(pkd + 2 * P.nbins + in);
              prefetch_l1(M.dd + (size_t)d * P.nbins + in);
            }
            if (lane >= 32 - kNM * 3) {
              // three lanes per mode: the run's anchor, the interval's coefficient rows and corrections
              const int k = (31 - lane) / 3, part = (31 - lane) % 3;
              const size_t sdk = sd + (size_t)k * M.n_det;
              const int jn = M.ch_iv[c + 1];
              if (part == 0)
                prefetch_l1(M.runs + (sdk * M.nchunks + c + 1) * 3);
              else if (part == 1)
                prefetch_l1(M.cg + (sdk * M.J + jn) * 8);
              else
                prefetch_l1(M.cbump + (sdk * M.J + jn) * 2);
            }
          }
        }
        if (kb < xb) {  // exact bins
          if (kStage) __syncwarp();
          continue;
        }
        const float4* rb = kStage ? &rbuf[wid][b][0] : nullptr;
        RunPhase r1;  // the run's anchor (single-mode plans: loaded once per run)
        if (kNM == 1) {
          const float4* ra = kStage ? rb + 104 : M.runs + (sd * M.nchunks + c) * 3;
          const float4 ra0 = ra[0], ra1 = ra[1];
          r1.x0 = ra0.x;
          r1.c0 = ra0.y;
          r1.s0 = ra0.z;
          r1.p1h = ra0.w;
          r1.p1l = ra1.x;
          r1.p2h = ra1.y;
          r1.p2l = ra1.z;
          r1.p3h = ra1.w;
          r1.p3l = ra[2].x;
        }
        if (kGrad && j != cur_iv) {
          if (cur_iv >= 0) flush_moments(mq, reinterpret_cast<float (*)[kMomPad]>(&msm[wid][0][0]), M.mom + (sd * M.J + cur_iv) * kNodeQ * kMoments, lane);
          cur_iv = j;
        }
        const int64_t i = (int64_t)kb + lane;
        if (lane < len && i < kcut) {
          float4 pk0, pk1, pk2;
          if (kStage) {
            pk0 = rb[lane];
            pk1 = rb[32 + lane];
            pk2 = rb[64 + lane];
          } else {
            const float4* pkd = M.pk + (size_t)d * 3 * P.nbins;
            pk0 = pkd[i];
            pk1 = pkd[P.nbins + i];
            pk2 = pkd[2 * P.nbins + i];
          }
          // the FP64 data norm of the weak-template form, loaded with the bin's
          // rows so that its latency overlaps theirs (2% on the gradient pass)
          const float2 Dn = M.dd[(size_t)d * P.nbins + i];
          const float t = pk2.w;
          const float u = (float)lane;
          const float u2 = u * u, u3 = u2 * u;
          // the model of each channel, summed over the modes of the bin
          float hrs[3] = {0.0f, 0.0f, 0.0f}, his[3] = {0.0f, 0.0f, 0.0f};
          float mx[3] = {0.0f, 0.0f, 0.0f};  // multi-mode: 2 Re h_k conj(sum of the earlier modes), per channel
          float cph = 0.0f, sph = 0.0f, xk = 0.0f, x2 = 0.0f;  // (single mode: used by the gradient)
#pragma unroll 1
          for (int k = 0; k < kNM; ++k) {
            const size_t sdk = sd + (size_t)k * M.n_det;
            RunPhase r = r1;
            if (kNM > 1) {
              const size_t v = (size_t)s * kNM + k;
              if (c >= M.nch[v] || i >= M.vcut[v]) continue;  // past the mode's range
              const float4* ra = M.runs + (sdk * M.nchunks + c) * 3;
              const float4 ra0 = ra[0], ra1 = ra[1];
              r.x0 = ra0.x;
              r.c0 = ra0.y;
              r.s0 = ra0.z;
              r.p1h = ra0.w;
              r.p1l = ra1.x;
              r.p2h = ra1.y;
              r.p2l = ra1.z;
              r.p3h = ra1.w;
              const float4 ra2 = ra[2];
              r.p3l = ra2.x;
              r.qx0 = ra2.y;
              r.qj = ra2.z;
            }
            // the straddled phase corner's term (multi-mode plans), added to the advance
            float qph = 0.0f;
            if (kNM > 1 && r.qj != 0.0f) {
              const float xq = fmaf(kSlope, u, r.qx0);
              if (xq > 0.0f) qph = r.qj * (xq * xq);
            }
            // explicit FMAs on the lnL path: the lnL and lnL+gradient instantiations must round alike.
            // The phase advance is summed error-free (reductions and sums keep their
            // roundings), its sine and cosine taken of the head and corrected to
            // first order in the tail.
            float del, dlo;
            {
              float ea, eb, ec;
              const float a = reduce_exact_ff(r.p1h * u, &ea), b = reduce_exact_ff(r.p2h * u2, &eb),
                          c = reduce_exact_ff(r.p3h * u3, &ec);
              float s1, t1, s2, t2, s3, t3;
              two_sum(a, b, s1, t1);
              two_sum(s1, c, s2, t2);
              two_sum(s2, fmaf(r.p1l, u, fmaf(r.p2l, u2, fmaf(r.p3l, u3, qph))), s3, t3);
              del = s3;
              dlo = ((ea + eb) + ec) + ((t1 + t2) + t3);
            }
            float sd_, cd_;
            sincos_poly(del, &sd_, &cd_);
            {
              const float sdc = fmaf(dlo, cd_, sd_);
              cd_ = fmaf(-dlo, sd_, cd_);
              sd_ = sdc;
            }
            cph = fmaf(r.c0, cd_, -(r.s0 * sd_));
            sph = fmaf(r.s0, cd_, r.c0 * sd_);
            // Renormalise the rotated phasor with one Newton step for 1/|e|
            // so that FP32 rounding leaves the model amplitude unbiased.
            const float m2 = fmaf(cph, cph, fmaf(sph, sph, -1.0f));  // |e|^2 - 1, one rounding
            const float corr = -0.5f * m2;
            cph = fmaf(corr, cph, cph);
            sph = fmaf(corr, sph, sph);
            {
              // TDI generation prefactor P(f): its zeros (f L = k/2) stay out of the
              // splines; with h = G (c - i s) the factor multiplies c - i s
              // explicit FMAs: the lnL and lnL+gradient kernels must round alike
              const float c2 = fmaf(pk2.y, cph, pk2.z * sph);
              const float s2 = fmaf(pk2.y, sph, -(pk2.z * cph));
              cph = c2;
              sph = s2;
            }
            // the interval's coefficient rows of this mode
            const float4* G = (kNM == 1 && kStage) ? rb + 96 : M.cg + (sdk * M.J + j) * 8;
            const float4 gl0 = G[6], gl1 = G[7];
            const float Glo[6] = {gl0.x, gl0.y, gl0.z, gl0.w, gl1.x, gl1.y};
            xk = fmaf(kSlope, u, r.x0);
            x2 = xk > 0.0f ? xk * xk : 0.0f;
            float kink[6];  // the amplitude kink and the midpoint correction of each quantity
            {
              const float4* BQ = (kNM == 1 && kStage) ? rb + 107 : M.cbump + (sdk * M.J + j) * 2;
              const float4 b0 = BQ[0], b1 = BQ[1];
              const float rr = t * (b1.z - t) * b1.w;
              const float r2 = rr * rr;
              kink[0] = b0.x * r2;
              kink[1] = b0.y * r2;
              kink[2] = b0.z * r2;
              kink[3] = b0.w * r2;
              kink[4] = b1.x * r2;
              kink[5] = b1.y * r2;
            }
            if (xk > 0.0f) {
              const float4* KF4 = reinterpret_cast<const float4*>(M.kinkF + sdk * 16);  // 64-byte aligned rows
              const float4 k0 = KF4[0], k1 = KF4[1], k2 = KF4[2], k3 = KF4[3];
              const float kfh[6] = {k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
              const float kfl[6] = {k2.x, k2.y, k2.z, k2.w, k3.x, k3.y};
              // multi-mode plans: intervals past the kink's own carry it in their coefficients
              const float g = (kNM == 1 || j == (int)k3.z) ? x2 : 0.0f;
#pragma unroll
              for (int q = 0; q < 6; ++q) kink[q] = fmaf(kfh[q], g, fmaf(kfl[q], g, kink[q]));
            }
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
              const float4 cr = G[2 * ch], ci = G[2 * ch + 1];
              const float gr = cr.x + (kink[2 * ch] + fmaf(t, fmaf(t, fmaf(t, cr.w, cr.z), cr.y), Glo[2 * ch]));
              const float gi = ci.x + (kink[2 * ch + 1] + fmaf(t, fmaf(t, fmaf(t, ci.w, ci.z), ci.y), Glo[2 * ch + 1]));
              const float hkr = fmaf(gr, cph, gi * sph), hki = fmaf(gi, cph, -(gr * sph));
              if (kNM > 1) mx[ch] = fmaf(2.0f, fmaf(hkr, hrs[ch], hki * his[ch]), mx[ch]);
              hrs[ch] += hkr;
              his[ch] += hki;
            }
          }
          float term = 0.0f;  // |d - h|^2 w
          float cross = 0.0f;  // (|h|^2 - 2 Re(d^* h)) w
          float hh = 0.0f;     // |h|^2 w
          float xdh = 0.0f;    // Re(d^* h) w
          float aphi = 0.0f;
          float ag[6];
          float mterm = 0.0f;
          float sqb = 0.0f;
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            const float hr = hrs[ch], hi = his[ch];
            const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
            const float2 dv = ch == 0 ? make_float2(pk0.x, pk0.y)
                                      : (ch == 1 ? make_float2(pk0.z, pk0.w) : make_float2(pk1.x, pk1.y));
            const float w = ch == 0 ? pk1.z : (ch == 1 ? pk1.w : pk2.x);
            const float er = dv.x - hr, ei = dv.y - hi;
            term = fmaf(fmaf(er, er, ei * ei), w, term);
            const float h2 = fmaf(hr, hr, hi * hi);
            hh = fmaf(h2, w, hh);
            {
              const float hw = h2 * w;
              const float a2 = fmaf(dv.x, dv.x, dv.y * dv.y) + (kNM > 1 ? h2 : 0.0f);
              sqb = fmaf(a2 * hw, w, sqb);
            }
            const float dh = fmaf(dv.x, hr, dv.y * hi);
            cross = fmaf(fmaf(-2.0f, dh, h2), w, cross);
            xdh = fmaf(dh, w, xdh);
            if (kNM > 1) mterm = fmaf(mx[ch], w, mterm);
            if (kMode == 2) model[off] = make_double2((double)hr / M.scale, (double)hi / M.scale);
            if (kGrad) {
              ag[2 * ch] = w * (er * cph - ei * sph);
              ag[2 * ch + 1] = w * (er * sph + ei * cph);
              aphi = fmaf(w, dv.x * hi - dv.y * hr, aphi);
            }
          }
          // Where the template is weaker than the residual, |d - h|^2 w =
          // |d|^2 w + (|h|^2 - 2 Re(d^* h)) w with the first term taken from
          // the FP64 data (float-float): the FP32 rounding then scales with
          // |h| instead of |d|, which matters when the data hold a loud signal.
          if (hh < term) {
            float t1, e1;
            two_sum(dsh, Dn.x, t1, e1);
            dsh = t1;
            dsl += e1 + Dn.y;
            term = cross;
          }
          // compensated accumulation
          const float yk = term - comp;
          const float tk = acc + yk;
          comp = (tk - acc) - yk;
          acc = tk;
          {
            const float yx = -2.0f * xdh - xcomp;
            const float tx = xacc + yx;
            xcomp = (tx - xacc) - yx;
            xacc = tx;
          }
          sqa += sqb;
          if (kNM > 1) {
            const float ym_ = mterm - mcomp;
            const float tm_ = macc + ym_;
            mcomp = (tm_ - macc) - ym_;
            macc = tm_;
          }
          if (kGrad && xk > 0.0f) {
            kinked = true;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
              km[q] = fmaf(ag[q], x2, km[q]);
              km[6 + q] = fmaf(ag[q], xk, km[6 + q]);
            }
          }
          if (kGrad) {
            const float tp[kMoments] = {1.0f, t, t * t, t * t * t};
#pragma unroll
            for (int p = 0; p < kMoments; ++p) {
              mq[0 * kMoments + p] = fmaf(aphi, tp[p], mq[0 * kMoments + p]);
#pragma unroll
              for (int qq = 0; qq < 6; ++qq) mq[(1 + qq) * kMoments + p] = fmaf(ag[qq], tp[p], mq[(1 + qq) * kMoments + p]);
            }
          }
        }
        if (kStage) __syncwarp();  // buffer b is refilled two runs on
      }
      if (kGrad && cur_iv >= 0) flush_moments(mq, reinterpret_cast<float (*)[kMomPad]>(&msm[wid][0][0]), M.mom + (sd * M.J + cur_iv) * kNodeQ * kMoments, lane);
      if (kGrad && __any_sync(0xffffffffu, kinked)) {
#pragma unroll
        for (int k = 0; k < 12; ++k) {
          float x = km[k];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          if (lane == 0) atomicAdd(M.kinkM + sd * 12 + k, x);
        }
      }
    }
  }
  // deterministic reduction: lanes (float-float) -> warps (FP64) -> block partial,
  // for the direct sum and the cross-term sum
  float vh, vl, xh, xl, mh, ml;
  two_sum(acc, -comp, vh, vl);
  two_sum(xacc, -xcomp, xh, xl);
  two_sum(macc, -mcomp, mh, ml);
  {
    float th, tl;
    two_sum(vh, dsh, th, tl);
    vh = th;
    vl += tl + dsl;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, vh, o);
    const float ol = __shfl_down_sync(0xffffffffu, vl, o);
    const float ph = __shfl_down_sync(0xffffffffu, xh, o);
    const float pl = __shfl_down_sync(0xffffffffu, xl, o);
    const float qh = __shfl_down_sync(0xffffffffu, mh, o);
    const float ql = __shfl_down_sync(0xffffffffu, ml, o);
    float th, tl;
    two_sum(vh, oh, th, tl);
    vh = th;
    vl += tl + ol;
    two_sum(xh, ph, th, tl);
    xh = th;
    xl += tl + pl;
    two_sum(mh, qh, th, tl);
    mh = th;
    ml += tl + ql;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sqa += __shfl_down_sync(0xffffffffu, sqa, o);
  if (lane == 0) {
    red[wid][0] = (double)vh + (double)vl;
    red[wid][1] = (double)xh + (double)xl;
    red[wid][2] = (double)mh + (double)ml;
    red[wid][3] = (double)sqa;
  }
  __syncthreads();
  if (threadIdx.x < kPartW) {
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < kMixThreads / 32; ++w) x += red[w][threadIdx.x];
    M.part[((size_t)s * M.nblk_dense + blockIdx.x) * kPartW + threadIdx.x] = x;
  }
}

// The float-float re-evaluation of the dense range of the samples that
// k_refine_select sends to it (rkind == kRefineFF): the dense stage's model
// (transfer splines with their midpoint corrections and kink, phase anchors,
// TDI prefactor, modes summed per bin), with every step from the spline
// coefficients to the residual |d - h|^2 w in float-float against
// float-float copies of the FP64 data, weights and prefactor.  The per-bin
// rounding falls from about 2e-7 of the terms to below 1e-13, so what is
// left of the error is the splines' own.  Same grid and run groups as
// k_dense_mixed; lane l of a warp first takes the phase anchor of the
// group's run l of every mode (shared memory), then each run takes a bin
// per lane.  Partials: fpart [B][nblk_dense].
template <int kNM>
__global__ void __launch_bounds__(kMixThreads) k_dense_ff(PlanDev P, MixedDev M,
                                                          const SampleBlock<double>* __restrict__ blocks) {
  __shared__ float4 anc[kMixThreads / 32][kNM][kChunkMax][2];  // ph0, ph1 | ph2, ph3 (hi, lo pairs)
  __shared__ int ancq[kMixThreads / 32][kNM][kChunkMax];        // the straddled phase corner, -1 when none
  __shared__ double red[kMixThreads / 32];
  const int s = blockIdx.y;
  if (M.rkind[s] != kRefineFF) return;  // uniform per block
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int first = (blockIdx.x * (kMixThreads / 32) + wid) * kChunkMax;
  int nc = M.nch[(size_t)s * kNM];
#pragma unroll
  for (int k = 1; k < kNM; ++k) nc = max(nc, M.nch[(size_t)s * kNM + k]);
  const int64_t kcut = blocks[s].kcut;
  FF acc = ff_make(0.0f, 0.0f);
  if (first < nc) {
    const int last = min(nc, first + kChunkMax);
    for (int d = 0; d < M.n_det; ++d) {
      const size_t sd = (size_t)s * kNM * M.n_det + d;  // (virtual sample of mode 0, detector)
      const int xb = M.xbind[sd];
      {
        const int c = first + lane;
#pragma unroll 1
        for (int k = 0; k < kNM; ++k) {
          const int v = s * kNM + k;
          float4 a0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), a1 = a0;
          int qk = -1;
          if (c < M.nch[v] && M.ch_begin[c] >= xb) {
            const AnchorFF A = run_anchor_ff(P, M, v, sd + (size_t)k * M.n_det, c, M.ch_begin[c], M.ch_iv[c]);
            a0 = make_float4(A.ph0.hi, A.ph0.lo, A.ph1.hi, A.ph1.lo);
            a1 = make_float4(A.ph2.hi, A.ph2.lo, A.ph3.hi, A.ph3.lo);
            qk = A.qk;
          }
          anc[wid][k][lane][0] = a0;
          anc[wid][k][lane][1] = a1;
          ancq[wid][k][lane] = qk;
        }
      }
      __syncwarp();
      for (int c = first; c < last; ++c) {
        const int kb = M.ch_begin[c];
        if (kb < xb) continue;  // exact bins
        const int j = M.ch_iv[c];
        const int64_t i = (int64_t)kb + lane;
        if (lane >= M.ch_len[c] || i >= kcut) continue;
        const FF f = ff_mulf(M.fstep_ff, (float)(P.k0 + i));  // k0 + i < 2^24: exact in FP32
        const float2 nfj = M.node_ff[j];
        const FF t = f - ff_make(nfj.x, nfj.y);
        const float tf = t.hi, u = (float)lane;
        FF hr[3], hi[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) hr[ch] = hi[ch] = ff_make(0.0f, 0.0f);
#pragma unroll 1
        for (int k = 0; k < kNM; ++k) {
          const int v = s * kNM + k;
          if (kNM > 1 && (c >= M.nch[v] || i >= M.vcut[v])) continue;  // past the mode's range
          const size_t sdk = sd + (size_t)k * M.n_det;
          const float4 a0 = anc[wid][k][c - first][0], a1 = anc[wid][k][c - first][1];
          FF ph = ff_make(a0.x, a0.y) + ff_mulf(ff_make(a0.z, a0.w), u);
          ph = ph + ff_mulf(ff_make(a1.x, a1.y), u * u);  // u^2, u^3 < 2^15: exact
          ph = ph + ff_mulf(ff_make(a1.z, a1.w), u * u * u);
          const float4 sa = M.sff[2 * v];
          const FF msf = ff_make(sa.z, sa.w);
          if (kNM > 1) {
            const int qk = ancq[wid][k][c - first];
            if (qk >= 0) {
              const float4 k4 = M.pkink[2 * v + qk];
              const FF xq = msf * f - ff_make(k4.x, k4.y);
              if (xq.hi > 0.0f) ph = ph + ff_make(k4.z, k4.w) * (xq * xq);
            }
          }
          FF sn, cs;
          dsincos(ff_wrap_2pi(ph), &sn, &cs);
          // the mode's transfer quantities on interval j: the spline (value and
          // slope coefficients in float-float), its midpoint correction, the kink
          const float4* G = M.cg + (sdk * M.J + j) * 8;
          const float4 gl0 = G[6], gl1 = G[7];
          const float alo[6] = {gl0.x, gl0.y, gl0.z, gl0.w, gl1.x, gl1.y};
          const float* blo = M.cgb + (sdk * M.J + j) * 6;
          const float4* BQ = M.cbump + (sdk * M.J + j) * 2;
          const float4 b0 = BQ[0], b1 = BQ[1];
          const float rr = tf * (b1.z - tf) * b1.w;
          const float r2 = rr * rr;
          const float bump[6] = {b0.x * r2, b0.y * r2, b0.z * r2, b0.w * r2, b1.x * r2, b1.y * r2};
          const float4* KF4 = reinterpret_cast<const float4*>(M.kinkF + sdk * 16);
          const float4 k0 = KF4[0], k1 = KF4[1], k2 = KF4[2], k3 = KF4[3];
          bool kinked = false;
          FF x2 = ff_make(0.0f, 0.0f);
          if (kNM == 1 || j == (int)k3.z) {
            const float4 sk = M.sff[2 * v + 1];
            const FF x = msf * f - ff_make(sk.x, sk.y);
            if (x.hi > 0.0f) {
              kinked = true;
              x2 = x * x;
            }
          }
          const float kfh[6] = {k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
          const float kfl[6] = {k2.x, k2.y, k2.z, k2.w, k3.x, k3.y};
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            FF g[2];
#pragma unroll
            for (int pp = 0; pp < 2; ++pp) {
              const int q = 2 * ch + pp;
              const float4 c4 = G[q];
              FF gq = ff_make(c4.x, alo[q]) + t * ff_addf(ff_make(c4.y, blo[q]), tf * fmaf(tf, c4.w, c4.z));
              gq = ff_addf(gq, bump[q]);
              if (kinked) gq = gq + ff_make(kfh[q], kfl[q]) * x2;
              g[pp] = gq;
            }
            // G e^{-i phase} = (g0 + i g1)(cos - i sin)
            hr[ch] = hr[ch] + (g[0] * cs + g[1] * sn);
            hi[ch] = hi[ch] + (g[1] * cs - g[0] * sn);
          }
        }
        // TDI prefactor, residual against the data, weight
        const float4* X = M.xff + (size_t)d * 6 * P.nbins + i;
        const float4 x3 = X[3 * (size_t)P.nbins], x4 = X[4 * (size_t)P.nbins], x5 = X[5 * (size_t)P.nbins];
        const FF pr = ff_make(x4.z, x4.w), pim = ff_make(x5.x, x5.y);
        const FF wch[3] = {ff_make(x3.x, x3.y), ff_make(x3.z, x3.w), ff_make(x4.x, x4.y)};
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          const float4 dv = X[(size_t)ch * P.nbins];
          const FF er = ff_make(dv.x, dv.y) - (hr[ch] * pr - hi[ch] * pim);
          const FF ei = ff_make(dv.z, dv.w) - (hr[ch] * pim + hi[ch] * pr);
          acc = acc + (er * er + ei * ei) * wch[ch];
        }
      }
      __syncwarp();  // the next detector's anchors overwrite this one's
    }
  }
  // lanes and warps in float-float, the block partial in FP64
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, acc.hi, o);
    const float ol = __shfl_down_sync(0xffffffffu, acc.lo, o);
    acc = acc + ff_make(oh, ol);
  }
  if (lane == 0) red[wid] = ff_to(acc);
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < kMixThreads / 32; ++w) x += red[w];
    M.fpart[(size_t)s * M.nblk_dense + blockIdx.x] = x;
  }
}

// sum |h|^2 w and sum |d|^2 w over the dense range [xbind, kcut) of each
// (sample, detector), one warp each.  On interval j the model's channel c is
// h_c = G_c(t) P(f) e^{-i phase} with G_c = a + b t + c t^2 + d t^3 (the
// transfer splines, re and im), plus C (X0 + Msec t)^2 past the amplitude
// peak (X0 = Msec f_j - Mf_peak), so |h_c|^2 w_c = |G_c(t)|^2 W_c and its sum
// over the interval's bins is sum_p g_p sum_k t_k^p W_c with g the
// coefficients of |G_c|^2: no per-bin rounding of the model.  Float-float on
// the FP32 pipes, in the interval's variable u = t / h (so that the moments
// sum u^p W stay in range); in FP64 this kernel bound the FP64 pipe.
constexpr int kHdThreads = 128;  // one block per (sample, detector), threads over its intervals
__device__ __forceinline__ FF hd_piece(const FF (&A)[6], const FF (&Bc)[6], const FF (&Cc)[6], const FF (&Dc)[6],
                                       const FF* Sm) {
  FF acc = ff_make(0.0f, 0.0f);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const int r = 2 * ch, i = 2 * ch + 1;
    const FF g0 = A[r] * A[r] + A[i] * A[i];
    const FF g1 = ff_mulf(A[r] * Bc[r] + A[i] * Bc[i], 2.0f);
    const FF g2 = (Bc[r] * Bc[r] + Bc[i] * Bc[i]) + ff_mulf(A[r] * Cc[r] + A[i] * Cc[i], 2.0f);
    const FF g3 = ff_mulf((A[r] * Dc[r] + A[i] * Dc[i]) + (Bc[r] * Cc[r] + Bc[i] * Cc[i]), 2.0f);
    const FF g4 = (Cc[r] * Cc[r] + Cc[i] * Cc[i]) + ff_mulf(Bc[r] * Dc[r] + Bc[i] * Dc[i], 2.0f);
    const FF g5 = ff_mulf(Cc[r] * Dc[r] + Cc[i] * Dc[i], 2.0f);
    const FF g6 = Dc[r] * Dc[r] + Dc[i] * Dc[i];
    const FF* m = Sm + ch * 7;
    acc = acc + ((g0 * m[0] + g1 * m[1]) + (g2 * m[2] + g3 * m[3]) + (g4 * m[4] + (g5 * m[5] + g6 * m[6])));
  }
  return acc;
}

__global__ void __launch_bounds__(kHdThreads) k_hd(PlanDev P, MixedDev M,
                                                  const SampleBlock<double>* __restrict__ blocks, int64_t B) {
  __shared__ double red[kHdThreads / 32][4];
  const int lane = threadIdx.x;
  const int64_t sd = blockIdx.x;  // (virtual sample, detector)
  if (sd >= B * M.n_modes * M.n_det) return;
  const int64_t v = sd / M.n_det;
  const int64_t s = v / M.n_modes;
  const int kmode = (int)(v % M.n_modes);
  const int d = (int)(sd % M.n_det);
  const SampleBlock<double>& b = blocks[s];
  double* out = M.hd + sd * kHdOut;
  // sum |d|^2 w over the sample's dense range [lo, kcut); sum |h|^2 w of the
  // mode over its own range [lo, vcut)
  const int64_t kcut = M.vcut[v];
  const int64_t lo = M.xbind[sd];
  if (b.status != kSampleOk || M.nsp[v] < 3 || lo >= kcut) {
    if (lane < kHdOut) out[lane] = 0.0;
    if (lane == 1 && b.status == kSampleOk && lo < b.kcut) {
      const double* ds = M.dsuf + (size_t)d * (P.nbins + 1);
      out[1] = ds[lo] - ds[b.kcut];
    }
    return;  // uniform per block
  }
  // the mode's amplitude kink point; multi-mode plans carry the kink in the
  // coefficients of the intervals after the one holding it (k_bump)
  const double Msec = b.wf.Msec, fpk = (M.hm && kmode > 0) ? M.hm[s].md[kmode].frA : b.wf.fpeak;
  const int jk = (int)M.kinkF[(size_t)sd * 16 + 14];
  // first bin with x = Msec f - Mf_peak > 0
  int64_t kpk = (int64_t)floor(fpk / (Msec * P.f_step)) - P.k0;
  for (int it = 0; it < 2 && kpk > 0 && Msec * ((double)(P.k0 + kpk - 1) * P.f_step) > fpk; ++it) --kpk;
  for (int it = 0; it < 2 && Msec * ((double)(P.k0 + kpk) * P.f_step) <= fpk; ++it) ++kpk;
  // intervals holding bins lo and kcut - 1
  auto iv_of = [&](int64_t k) {
    int a = 0, z = M.J - 2;
    while (a < z) {
      const int mid = (a + z + 1) >> 1;
      if (M.iv_first[mid] <= k) a = mid; else z = mid - 1;
    }
    return a;
  };
  const int jlo = iv_of(lo), jhi = iv_of(kcut - 1);
  // the kink coefficients C_q, Msec and the kink point in float-float
  const float* kf = M.kinkF + (size_t)sd * 16;
  FF KC[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) KC[q] = ff_make(kf[2 + q], kf[8 + q]);
  const float4 sa = M.sff[2 * v], sk = M.sff[2 * v + 1];
  const FF msf = ff_make(sa.z, sa.w), fpf = ff_make(sk.x, sk.y);
  const FF* wm = M.wmom + (size_t)d * P.nbins * kMomStride;
  const FF* ym = M.ym + (size_t)sd * 7 * M.J;
  FF sum = ff_make(0.0f, 0.0f);
  float eh = 0.0f, eha = 0.0f;
  for (int j = jlo + lane; j <= jhi; j += kHdThreads) {
    const int64_t e1 = M.iv_first[j], e2 = M.iv_first[j + 1];
    const int64_t k1 = max(e1, lo), k2 = min(e2, kcut);
    if (k1 >= k2) continue;
    const FF* tot = M.wtot + ((size_t)d * M.J + j) * kMomStride;
    auto F = [&](int64_t k, int idx) { return k >= e2 ? tot[idx] : wm[(size_t)k * kMomStride + idx]; };
    // the spline coefficients in the interval's own variable u = t / h (the
    // moments are sums of u^p W): A, B h, C h^2, D h^3
    const FF h = M.gff[j], h2 = h * h, h3 = h2 * h;
    FF A[6], Bc[6], Cc[6], Dc[6];
    const float4* cg = M.cg + ((size_t)sd * M.J + j) * 8;
    const float* alo = reinterpret_cast<const float*>(cg + 6);
    const float* blo = M.cgb + ((size_t)sd * M.J + j) * 6;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float4 c4 = cg[q];
      A[q] = ff_make(c4.x, alo[q]);
      Bc[q] = ff_make(c4.y, blo[q]) * h;
      Cc[q] = ff_mulf(h2, c4.z);
      Dc[q] = ff_mulf(h3, c4.w);
    }
    // the splines' error at the midpoint (kink-free values on both sides, or
    // both with the kink in a folded interval)
    const bool folded = jk >= 0 && j > jk;
    const float2 nfj = M.node_ff[j];
    const FF X0 = msf * ff_make(nfj.x, nfj.y) - fpf;
    const FF K = msf * h;  // Msec h: x = X0 + K u
    const FF Xm = X0 + ff_mulf(K, 0.5f);
    const FF Xm2 = Xm * Xm;
    float delta[6], gm[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const FF sp = A[q] + ff_mulf(Bc[q] + ff_mulf(Cc[q] + ff_mulf(Dc[q], 0.5f), 0.5f), 0.5f);
      FF ex = ym[(size_t)q * M.J + j];
      if (folded) ex = ex + KC[q] * Xm2;
      delta[q] = (ex - sp).hi;
      gm[q] = (Xm.hi > 0.0f && !folded) ? (ex + KC[q] * Xm2).hi : ex.hi;
    }
    FF Sm[21];
    // [k1, ks) without the kink term, [ks, k2) with it (folded intervals hold it already)
    const int64_t ks = folded ? k2 : min(max(kpk, k1), k2);
    if (ks > k1) {
#pragma unroll
      for (int x = 0; x < 21; ++x) Sm[x] = F(ks, x) - F(k1, x);
      sum = sum + hd_piece(A, Bc, Cc, Dc, Sm);
    }
    if (ks < k2) {
      // C (X0 + K u)^2 = C X0^2 + 2 C X0 K u + C K^2 u^2
      const FF X02 = X0 * X0, X0K2 = ff_mulf(X0 * K, 2.0f), K2 = K * K;
      FF A2[6], B2[6], C2[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        A2[q] = A[q] + KC[q] * X02;
        B2[q] = Bc[q] + KC[q] * X0K2;
        C2[q] = Cc[q] + KC[q] * K2;
      }
#pragma unroll
      for (int x = 0; x < 21; ++x) Sm[x] = F(k2, x) - F(ks, x);
      sum = sum + hd_piece(A2, B2, C2, Dc, Sm);
    }
    // first-order change of sum |h|^2 w over the interval if the splines' error
    // had the shape 16 u^2 (1 - u)^2 times its midpoint value
    if (!M.wspike[(size_t)d * M.J + j]) {
      float e = 0.0f;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const float m2 = (F(k2, ch * 7 + 2) - F(k1, ch * 7 + 2)).hi, m3 = (F(k2, ch * 7 + 3) - F(k1, ch * 7 + 3)).hi,
                    m4 = (F(k2, ch * 7 + 4) - F(k1, ch * 7 + 4)).hi;
        const float bump = 16.0f * (m2 - 2.0f * m3 + m4);
        e += 2.0f * (gm[2 * ch] * delta[2 * ch] + gm[2 * ch + 1] * delta[2 * ch + 1]) * bump;
      }
      eh += e;
      eha += fabsf(e);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum = sum + ff_make(__shfl_xor_sync(0xffffffffu, sum.hi, o), __shfl_xor_sync(0xffffffffu, sum.lo, o));
    eh += __shfl_xor_sync(0xffffffffu, eh, o);
    eha += __shfl_xor_sync(0xffffffffu, eha, o);
  }
  if ((lane & 31) == 0) {
    red[lane >> 5][0] = ff_to(sum);
    red[lane >> 5][1] = 0.0;
    red[lane >> 5][2] = (double)eh;
    red[lane >> 5][3] = (double)eha;
  }
  __syncthreads();
  if (lane == 0) {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kHdThreads / 32; ++w)
      for (int q = 0; q < 4; ++q) t[q] += red[w][q];
    const double* ds = M.dsuf + (size_t)d * (P.nbins + 1);
    out[0] = t[0];
    out[1] = ds[lo] - ds[b.kcut];
    out[2] = t[1];
    out[3] = t[2];
    out[4] = t[3];
    out[5] = 0.0;
  }
}

__global__ void k_mixed_finalize(PlanDev P, MixedDev M, const SampleBlock<double>* __restrict__ blocks, int64_t B,
                                 double* __restrict__ lnl, int32_t* __restrict__ status) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  const SampleBlock<double>& b = blocks[s];
  if (b.status != kSampleOk) {
    lnl[s] = -INFINITY;
    if (status) status[s] = b.status;
    return;
  }
  // dense bins: the direct sum of |d - h|^2 w, or the split form for templates
  // far from the data (residual above 2 sqrt(<h|h> <d|d>)), where the FP32
  // rounding of the model enters only the cross term
  double R = 0.0, X = 0.0, H = 0.0, Dd = 0.0, Cm = 0.0;
  for (int k = 0; k < M.nblk_dense; ++k) {
    R += M.part[((size_t)s * M.nblk_dense + k) * kPartW];
    X += M.part[((size_t)s * M.nblk_dense + k) * kPartW + 1];
    Cm += M.part[((size_t)s * M.nblk_dense + k) * kPartW + 2];
  }
  if (M.n_modes > 1) {
    // multi-mode plans: the split form for far templates with sum |h|^2 w =
    // the modes' own sums (exact, from their splines) + their cross terms
    // (dense stage)
    for (int k = 0; k < M.n_modes; ++k)
      for (int d = 0; d < M.n_det; ++d) {
        const double* hv = M.hd + (((size_t)s * M.n_modes + k) * M.n_det + d) * kHdOut;
        H += hv[0] + hv[3];
      }
    for (int d = 0; d < M.n_det; ++d) Dd += M.hd[((size_t)s * M.n_modes * M.n_det + d) * kHdOut + 1];
    const double Ht = H + Cm;
    double acc = (R > 2.0 * sqrt(fmax(Ht, 0.0) * Dd)) ? (Dd + X) + Ht : R;
    if (M.rkind[s] == kRefineExact) {  // the exact re-evaluation of the dense range
      acc = 0.0;
      for (int k = 0; k < M.rblocks; ++k) acc += M.rpart[(size_t)s * M.rblocks + k];
    } else if (M.rkind[s] == kRefineFF) {  // the float-float one
      acc = 0.0;
      for (int k = 0; k < M.nblk_dense; ++k) acc += M.fpart[(size_t)s * M.nblk_dense + k];
    }
    if (M.xbin[s * M.n_modes] > 0)
      for (int k = 0; k < M.xblocks; ++k) acc += M.xpart[(size_t)s * M.xblocks + k];
    for (int k = 0; k < M.zblocks; ++k) acc += M.zpart[(size_t)s * M.zblocks + k];
    const double v = -2.0 * P.df * (acc + P.suffix[b.kcut]);
    lnl[s] = v;
    if (status) status[s] = isfinite(v) ? kSampleOk : kSampleNonFinite;
    return;
  }
  for (int d = 0; d < M.n_det; ++d) {
    // sum |h|^2 w from the splines, corrected by the midpoint estimate of their error
    H += M.hd[((size_t)s * M.n_det + d) * kHdOut] + M.hd[((size_t)s * M.n_det + d) * kHdOut + 3];
    Dd += M.hd[((size_t)s * M.n_det + d) * kHdOut + 1];
  }
  double acc = (R > 2.0 * sqrt(H * Dd)) ? (Dd + X) + H : R;
  if (M.rkind[s] == kRefineExact) {  // the exact re-evaluation of the dense range
    acc = 0.0;
    for (int k = 0; k < M.rblocks; ++k) acc += M.rpart[(size_t)s * M.rblocks + k];
  } else if (M.rkind[s] == kRefineFF) {  // the float-float one
    acc = 0.0;
    for (int k = 0; k < M.nblk_dense; ++k) acc += M.fpart[(size_t)s * M.nblk_dense + k];
  }
  if (M.xbin[s] > 0)
    for (int k = 0; k < M.xblocks; ++k) acc += M.xpart[(size_t)s * M.xblocks + k];
  for (int k = 0; k < M.zblocks; ++k) acc += M.zpart[(size_t)s * M.zblocks + k];
  const double v = -2.0 * P.df * (acc + P.suffix[b.kcut]);
  lnl[s] = v;
  if (status) status[s] = isfinite(v) ? kSampleOk : kSampleNonFinite;
}

__global__ void k_mixed_grad_finalize(MixedDev M, int64_t B, double xscale, double* __restrict__ grad) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  const bool ok = reinterpret_cast<const SampleBlock<GradScalar>*>(M.gblocks)[s].status == kSampleOk;
  const bool exact = M.xbin[s] > 0;
  for (int p = 0; p < 11; ++p) {
    double acc = 0.0;
    if (ok) {
      for (int d = 0; d < M.n_det; ++d) {
        for (int b = 0; b < M.nblk_sparse; ++b) acc += M.gpart[(((size_t)s * M.n_det + d) * M.nblk_sparse + b) * 11 + p];
        if (p == 10) acc += M.gdir[(size_t)s * M.n_det + d];
      }
      double x = 0.0;
      if (exact)
        for (int b = 0; b < M.xblocks; ++b) x += M.xgpart[((size_t)s * M.xblocks + b) * 11 + p];
      for (int b = 0; b < M.zblocks; ++b) x += M.zgpart[((size_t)s * M.zblocks + b) * 11 + p];
      acc += xscale * x;
    }
    grad[11 * s + p] = acc;
  }
}

// ------------------------------------------------------------------ data ingestion
__global__ void k_mixed_ingest(PlanDev P, MixedDev M, int det, const double2* __restrict__ data,
                               const double* __restrict__ psd) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nbins) return;
  double dd = 0.0;
  float dr[3], di[3], wf[3];
  FF wff[3];
  float4* X = M.xff + (size_t)det * 6 * P.nbins + i;
  const bool zw = in_zero_window(M, det, i);  // evaluated exactly: no weight in the dense stage
  for (int ch = 0; ch < 3; ++ch) {
    const double2 v = data[ch * P.nbins + i];
    const FF re = ff_from(v.x * M.scale), im = ff_from(v.y * M.scale);
    dr[ch] = re.hi;
    di[ch] = im.hi;
    X[(size_t)ch * P.nbins] = make_float4(re.hi, re.lo, im.hi, im.lo);
    const bool on = ((P.chan_mask >> ch) & 1) && !zw;
    wff[ch] = on ? ff_from(1.0 / (psd[ch * P.nbins + i] * M.scale * M.scale)) : ff_make(0.0f, 0.0f);
    wf[ch] = wff[ch].hi;
    if (on) dd += (v.x * v.x + v.y * v.y) / psd[ch * P.nbins + i];
  }
  const float hi = (float)dd;
  M.dd[(size_t)det * P.nbins + i] = make_float2(hi, (float)(dd - (double)hi));
  M.wrow[i] = dd;
  const TdiFactor tf = P.tdi[(size_t)det * P.nbins + i];
  float4* pk = M.pk + (size_t)det * 3 * P.nbins;
  pk[i] = make_float4(dr[0], di[0], dr[1], di[1]);
  pk[P.nbins + i] = make_float4(dr[2], di[2], wf[0], wf[1]);
  pk[2 * P.nbins + i] = make_float4(wf[2], (float)tf.pre, (float)tf.pim, M.bin_t[i]);
  const FF pre = ff_from(tf.pre), pim = ff_from(tf.pim);
  X[3 * (size_t)P.nbins] = make_float4(wff[0].hi, wff[0].lo, wff[1].hi, wff[1].lo);
  X[4 * (size_t)P.nbins] = make_float4(wff[2].hi, wff[2].lo, pre.hi, pre.lo);
  X[5 * (size_t)P.nbins] = make_float4(pim.hi, pim.lo, 0.0f, 0.0f);
}

// Within-interval weight moments of detector det (set-up): one thread per
// (interval, channel) runs over the interval's bins in order, writing the
// exclusive prefix sums of u^p W_c (p = 0..6) at every bin and the interval's
// totals; W_c = w_c |P|^2 / scale^2, u = (f_k - f_j) / h_j; summed in FP64,
// stored as float-float.
// per interval of one detector: does the weight sum_c w_c |P|^2 spike (its
// largest bin above kSpikeRatio times the interval's mean)?
__global__ void k_wspike(PlanDev P, MixedDev M, int det, int32_t* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M.J) return;
  int flag = 0;
  if (j < M.J - 1) {
    const int64_t k1 = M.iv_first[j], k2 = M.iv_first[j + 1];
    double mx = 0.0, sum = 0.0;
    for (int64_t k = k1; k < k2; ++k) {
      if (in_zero_window(M, det, k)) continue;
      const TdiFactor tf = P.tdi[(size_t)det * P.nbins + k];
      double w = 0.0;
      for (int c = 0; c < 3; ++c) w += P.w[((size_t)det * 3 + c) * P.nbins + k];
      w *= tf.pre * tf.pre + tf.pim * tf.pim;
      mx = fmax(mx, w);
      sum += w;
    }
    flag = k2 > k1 && mx > kSpikeRatio * sum / (double)(k2 - k1);
  }
  out[(size_t)det * M.J + j] = flag;
}

__global__ void k_wmoments(PlanDev P, MixedDev M, int det, FF* __restrict__ wmom, FF* __restrict__ wtot) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (M.J - 1) * 3) return;
  const int j = t / 3, c = t % 3;
  const int64_t k1 = M.iv_first[j], k2 = M.iv_first[j + 1];
  const double fj = M.node_f[j];
  const double is2 = 1.0 / (M.scale * M.scale);
  double acc[7];
#pragma unroll
  for (int p = 0; p < 7; ++p) acc[p] = 0.0;
  FF* pm = wmom + (size_t)det * P.nbins * kMomStride + c * 7;
  const double ih = 1.0 / M.gh[j];
  for (int64_t k = k1; k < k2; ++k) {
    const double tk = ((double)(P.k0 + k) * P.f_step - fj) * ih;
    const TdiFactor tf = P.tdi[(size_t)det * P.nbins + k];
    const size_t off = ((size_t)det * 3 + c) * P.nbins + k;
    const double w = in_zero_window(M, det, k) ? 0.0 : P.w[off];
    double tp = w * (tf.pre * tf.pre + tf.pim * tf.pim) * is2;
#pragma unroll
    for (int p = 0; p < 7; ++p) {
      pm[(size_t)k * kMomStride + p] = ff_from(acc[p]);
      acc[p] += tp;
      tp *= tk;
    }
  }
  FF* tot = wtot + ((size_t)det * M.J + j) * kMomStride + c * 7;
#pragma unroll
  for (int p = 0; p < 7; ++p) tot[p] = ff_from(acc[p]);
}

// ------------------------------------------------------------------ host side
template <class X>
static int alloc(MixedBuffers* mb, X** ptr, size_t count) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(X) * (count ? count : 1));
  if (e != cudaSuccess) {
    set_error("mixed plan: cudaMalloc of %zu bytes failed: %s", sizeof(X) * count, cudaGetErrorString(e));
    return PES_ENOMEM;
  }
  mb->allocs.push_back(p);
  *ptr = reinterpret_cast<X*>(p);
  return PES_OK;
}

// Spline fit of the first B samples: staged register-segment kernels (phase
// systems in FF, transfer systems in FP32), or the global-scratch kernel for
// grids beyond 64 x 32 intervals.
// The phase systems on st_phase, the transfer systems on st_transfer (the
// same stream, or a second one so that the two fits overlap).
static void launch_spline_fit(const MixedDev& M, int64_t B, cudaStream_t st_phase, cudaStream_t st_transfer) {
  const int64_t nsd = B * M.n_det;
  const int seg = spline_seg(M.J);
  if (seg == 0) {
    k_spline_fit_wide<<<(unsigned)nsd, kSplineThreads, 0, st_phase>>>(M);
    return;
  }
  const unsigned bp = (unsigned)ceil_div(nsd, (int64_t)kFitWarps);
  const unsigned bt = (unsigned)ceil_div(nsd * 6, (int64_t)kFitWarps);
  if (seg == 32) {
    k_spline_fit<32, FF><<<bp, kFitWarps * 32, fit_smem_bytes<FF, true>(M.J), st_phase>>>(M, nsd);
    k_spline_fit<32, float><<<bt, kFitWarps * 32, fit_smem_bytes<float, true>(M.J), st_transfer>>>(M, nsd * 6);
  } else {
    k_spline_fit<kSegMax, FF><<<bp, kFitWarps * 32, fit_smem_bytes<FF, false>(M.J), st_phase>>>(M, nsd);
    k_spline_fit<kSegMax, float><<<bt, kFitWarps * 32, fit_smem_bytes<float, false>(M.J), st_transfer>>>(M,
                                                                                                       nsd * 6);
  }
}

int mixed_create(PesPlan* p) {
  const PesPlanDesc& d = p->desc;
  PES_REQUIRE(d.n_sparse >= 8 && d.n_sparse <= 65536, "mixed plan: n_sparse must be 8..65536, got %d", d.n_sparse);
  PES_REQUIRE(d.k0 >= 1, "mixed plan: the grid must start above 0 Hz (k0 >= 1)");
  PES_REQUIRE(d.k0 + d.nbins < (int64_t)1 << 24, "mixed plan: bin indices k0 + i must stay below 2^24");
  PES_REQUIRE(d.nbins >= 8, "mixed plan: needs at least 8 bins");
  MixedBuffers* mb = new MixedBuffers();
  p->mixed = mb;
  {
    // highest priority: the side kernels are few, long-latency blocks that should
    // get SM slots as soon as the main stream's blocks retire
    int least = 0, greatest = 0;
    PES_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    PES_CHECK_CUDA(cudaStreamCreateWithPriority(&mb->side, cudaStreamNonBlocking, greatest));
  }
  PES_CHECK_CUDA(cudaEventCreateWithFlags(&mb->fork, cudaEventDisableTiming));
  PES_CHECK_CUDA(cudaEventCreateWithFlags(&mb->join, cudaEventDisableTiming));
  PES_CHECK_CUDA(cudaEventCreateWithFlags(&mb->xready, cudaEventDisableTiming));
  PES_CHECK_CUDA(cudaStreamCreateWithFlags(&mb->aux, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&mb->ev_nodes, &mb->ev_tfit, &mb->ev_dense, &mb->ev_tadj, &mb->ev_hd, &mb->ev_pfit,
                         &mb->ev_kink, &mb->ev_xgrad})
    PES_CHECK_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  MixedDev& M = mb->dev;
  const int64_t n = d.nbins;
  const int J = d.n_sparse;
  const int nd = d.n_det;
  const int64_t B = d.max_batch;
  M.J = J;
  M.n_det = nd;
  M.n_modes = d.approximant == PES_APPROX_PHENOMHM ? kHMModes : 1;
  M.hm = hm_blocks<double>(p);
  const int64_t V = B * M.n_modes;  // virtual samples (sample, mode)
  if (spline_seg(J) == 32) {
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_fit<32, FF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)fit_smem_bytes<FF, true>(J)));
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_fit<32, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)fit_smem_bytes<float, true>(J)));
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_adjoint_staged<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)adj_smem_bytes<double>(J)));
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_adjoint_staged<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)adj_smem_bytes<float>(J)));
  } else if (spline_seg(J) == kSegMax) {
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_fit<kSegMax, FF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)fit_smem_bytes<FF, false>(J)));
    PES_CHECK_CUDA(cudaFuncSetAttribute(k_spline_fit<kSegMax, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)fit_smem_bytes<float, false>(J)));
  }
  M.scale = 3.085677581491367e16 / (1.476625038050124729627979840144936351e3 * 4.925490947641266978197229498498379006e-6);
  M.scale_ff = ff_from(M.scale);
  mb->stage_grad = (size_t)nd * (size_t)n * 3 * sizeof(float4) > ((size_t)64 << 20);
  if (const char* env = std::getenv("PES_DENSE_STAGE")) {  // "1": always stage, "0": never
    if (env[0] == '1') mb->stage_grad = true;
    if (env[0] == '0') mb->stage_grad = false;
  }
  M.scale_f = (float)M.scale;
  M.fstep_ff = ff_from(d.f_step);
  M.f_step = d.f_step;
  for (int k = 0; k < nd; ++k) mb->gen.gen20[k] = d.det[k].generation == 20;
  // shared sparse grid, bin -> interval map, runs
  const double flo = (double)d.k0 * d.f_step, fhi = (double)(d.k0 + n - 1) * d.f_step;
  std::vector<double> nf(J);
  for (int j = 0; j < J; ++j) nf[j] = flo * std::pow(fhi / flo, (double)j / (J - 1));
  nf[0] = flo;
  nf[J - 1] = fhi;
  std::vector<float> bt(n);
  std::vector<int32_t> cb, cl, ci;
  std::vector<int32_t> ivf(J + 1, (int32_t)n);
  int j = 0;
  int run_iv = -1, run_len = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double f = (double)(d.k0 + i) * d.f_step;
    while (j + 1 < J - 1 && nf[j + 1] <= f) ++j;
    for (int jj = j; jj >= 0 && ivf[jj] == (int32_t)n; --jj) ivf[jj] = (int32_t)i;
    bt[i] = (float)(f - nf[j]);
    if (j != run_iv || run_len == kChunkMax) {
      cb.push_back((int32_t)i);
      cl.push_back(0);
      ci.push_back(j);
      run_iv = j;
      run_len = 0;
    }
    cl.back() += 1;
    run_len += 1;
  }
  // fastest orbital angular frequency: the yearly revolution, or a geocentric
  // constellation's rotation about the Earth (TianQin: 3.65 days)
  M.xblocks = kExactBlocks;
  for (int k = 0; k < PES_MAX_DETECTORS; ++k) M.omega[k] = 0.0;
  for (int k = 0; k < nd; ++k) {
    M.omega[k] = std::fabs(d.det[k].orbit.omega_revolution);
    if (d.det[k].orbit.kind == 1) {
      M.omega[k] = std::max(M.omega[k], std::fabs(d.det[k].orbit.omega_rotation));
      M.xblocks = kExactBlocksGeo;
    }
  }
  M.nchunks = (int32_t)cb.size();
  M.nblk_dense = (int32_t)ceil_div(M.nchunks, (long long)kChunkMax * (kMixThreads / 32));
  M.nblk_sparse = (int32_t)ceil_div(J, kSparseThreads);
  int rc = PES_OK;
  double *node_f = nullptr, *scr, *part, *gpart, *gdir;
  float* ybar;
  FF *yv, *cphi, *gff;
  float *mom, *kM;
  double *gh, *ginvh, *glo, *gup, *ginvden, *gcp;
  float* gf;
  TdiFactor* tdn;
  float4* tdn_ff;
  float4* sff;
  unsigned long long* cfrac;
  float2* node_ff;
  int32_t *chb, *chl, *chi, *nsp, *nch, *xbin, *xbind, *ivfirst, *vcut, *wspk;
  double *xpart, *xgpart;
  FF *wmom, *wtot;
  double *dsuf, *wrow, *hdv, *rpart, *fpart;
  int32_t* rkind;
  float4* xff;
  float* cgb;
  float2* mid_ff;
  float4* tdm_ff;
  FF* ymv;
  float4* cbump;
  SampleBlock<GradScalar>* gblk;
  double *kR, *kC;
  float* kF;
  float* bin_t;
  float4* runs;
  float4* pk;
  float2* ddv;
  float4* cg;
  const size_t sd = (size_t)V * nd;  // per (virtual sample, detector)
  // multi-mode plans: lnL only (no gradient buffers)
  const bool multi = M.n_modes > 1;
  const size_t gsd = multi ? 1 : sd;
  const size_t wn = (size_t)nd * n * kMomStride, wj = (size_t)nd * J * kMomStride;
  if ((rc = alloc(mb, &node_f, J)) || (rc = alloc(mb, &chb, M.nchunks)) || (rc = alloc(mb, &chl, M.nchunks)) ||
      (rc = alloc(mb, &chi, M.nchunks)) || (rc = alloc(mb, &bin_t, n)) ||
      (rc = alloc(mb, &runs, sd * M.nchunks * 3)) || (rc = alloc(mb, &pk, (size_t)nd * 3 * n)) || (rc = alloc(mb, &ddv, (size_t)nd * n)) || (rc = alloc(mb, &nsp, V)) || (rc = alloc(mb, &nch, V)) || (rc = alloc(mb, &vcut, V)) ||
      (rc = alloc(mb, &yv, sd * kNodeQ * J)) || (rc = alloc(mb, &scr, sd * kNodeQ * J)) ||
      (rc = alloc(mb, &gh, J)) || (rc = alloc(mb, &ginvh, J)) || (rc = alloc(mb, &glo, J)) ||
      (rc = alloc(mb, &gup, J)) || (rc = alloc(mb, &ginvden, J)) || (rc = alloc(mb, &gcp, J)) ||
      (rc = alloc(mb, &gf, (size_t)kGfCount * J)) || (rc = alloc(mb, &gff, (size_t)kGfCount * J)) || (rc = alloc(mb, &tdn, (size_t)nd * J)) || (rc = alloc(mb, &tdn_ff, (size_t)nd * J)) || (rc = alloc(mb, &sff, (size_t)2 * V)) ||
      (rc = alloc(mb, &cfrac, (size_t)V)) || (rc = alloc(mb, &node_ff, J)) ||
      (rc = alloc(mb, &cphi, sd * J * 4)) || (rc = alloc(mb, &cg, sd * J * 8)) ||
      (rc = alloc(mb, &mom, gsd * J * kNodeQ * kMoments)) || (rc = alloc(mb, &ybar, gsd * kNodeQ * J)) ||
      (rc = alloc(mb, &part, (size_t)B * M.nblk_dense * kPartW)) ||
      (rc = alloc(mb, &wmom, wn)) || (rc = alloc(mb, &wtot, wj)) ||
      (rc = alloc(mb, &dsuf, (size_t)nd * (n + 1))) || (rc = alloc(mb, &wrow, (size_t)n)) ||
      (rc = alloc(mb, &cgb, sd * J * 6)) || (rc = alloc(mb, &hdv, sd * kHdOut)) ||
      (rc = alloc(mb, &mid_ff, J)) || (rc = alloc(mb, &tdm_ff, (size_t)nd * J)) || (rc = alloc(mb, &ymv, sd * 7 * J)) ||
      (rc = alloc(mb, &cbump, sd * J * 2)) || (rc = alloc(mb, &wspk, (size_t)nd * J)) ||
      (rc = alloc(mb, &rpart, (size_t)B * kRefineBlocks)) || (rc = alloc(mb, &rkind, (size_t)B)) ||
      (rc = alloc(mb, &fpart, (size_t)B * M.nblk_dense)) || (rc = alloc(mb, &xff, (size_t)nd * 6 * n)) ||
      (rc = alloc(mb, &gpart, gsd * M.nblk_sparse * 11)) || (rc = alloc(mb, &gdir, gsd)) ||
      (rc = alloc(mb, &gblk, (size_t)B)) || (rc = alloc(mb, &kR, sd * 6)) || (rc = alloc(mb, &kC, sd * 6)) ||
      (rc = alloc(mb, &kF, sd * 16)) || (rc = alloc(mb, &kM, gsd * 12)) || (rc = alloc(mb, &xbin, V)) || (rc = alloc(mb, &xbind, sd)) ||
      (rc = alloc(mb, &ivfirst, J + 1)) || (rc = alloc(mb, &xpart, (size_t)B * M.xblocks)) ||
      (rc = alloc(mb, &xgpart, (size_t)B * M.xblocks * 11)))
    return rc;
  PES_CHECK_CUDA(cudaMemcpy(ivfirst, ivf.data(), sizeof(int32_t) * (J + 1), cudaMemcpyHostToDevice));
  PES_CHECK_CUDA(cudaMemset(xbin, 0, sizeof(int32_t) * V));
  PES_CHECK_CUDA(cudaMemset(xbind, 0, sizeof(int32_t) * sd));
  PES_CHECK_CUDA(cudaMemcpy(node_f, nf.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
  {
    std::vector<float2> nff(J);
    for (int jj = 0; jj < J; ++jj) {
      const FF v = ff_from(nf[jj]);
      nff[jj] = make_float2(v.hi, v.lo);
    }
    PES_CHECK_CUDA(cudaMemcpy(node_ff, nff.data(), sizeof(float2) * J, cudaMemcpyHostToDevice));
  }
  {
    std::vector<TdiFactor> tf((size_t)nd * J);
    std::vector<float4> tff((size_t)nd * J);
    for (int k = 0; k < nd; ++k)
      for (int jj = 0; jj < J; ++jj) {
        Cx<double> D, Pf;
        tdi_factors(nf[jj], d.det[k].orbit.arm_sec, d.det[k].generation == 20, D, Pf);
        (void)Pf;  // the generation prefactor P(f) is applied per bin, outside the splines
        tf[(size_t)k * J + jj] = TdiFactor{D.re, D.im, 1.0, 0.0};
        const FF re = ff_from(D.re), im = ff_from(D.im);
        tff[(size_t)k * J + jj] = make_float4(re.hi, re.lo, im.hi, im.lo);
      }
    PES_CHECK_CUDA(cudaMemcpy(tdn, tf.data(), sizeof(TdiFactor) * tf.size(), cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(tdn_ff, tff.data(), sizeof(float4) * tff.size(), cudaMemcpyHostToDevice));
  }
  for (int k = 0; k < PES_MAX_DETECTORS; ++k) {
    M.orbit_ff[k] = orbit_ff(k < nd ? d.det[k].orbit : d.det[0].orbit);
    M.orbit_f[k] = orbit_f(k < nd ? d.det[k].orbit : d.det[0].orbit);
  }
  {
    // shared not-a-knot system of the node grid: rows 1..J-2 with the first-row
    // elimination and without the last-row one (that row depends on the sample)
    std::vector<double> h(J, 0.0), ih(J, 0.0), lo(J, 0.0), up(J, 0.0), iden(J, 0.0), cp(J, 0.0);
    for (int i = 0; i + 1 < J; ++i) {
      h[i] = nf[i + 1] - nf[i];
      ih[i] = 1.0 / h[i];
    }
    double cprev = 0.0;
    for (int i = 1; i + 1 < J; ++i) {
      const double h0 = h[i - 1], h1 = h[i];
      double l = h0, dgl = 2.0 * (h0 + h1), u = h1;
      if (i == 1) {
        dgl += h0 * (h0 + h1) / h1;
        u -= h0 * h0 / h1;
        l = 0.0;
      }
      const double den = dgl - l * cprev;
      lo[i] = l;
      up[i] = u;
      iden[i] = 1.0 / den;
      cp[i] = u / den;
      cprev = cp[i];
    }
    PES_CHECK_CUDA(cudaMemcpy(gh, h.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(ginvh, ih.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(glo, lo.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(gup, up.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(ginvden, iden.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(gcp, cp.data(), sizeof(double) * J, cudaMemcpyHostToDevice));
    std::vector<float> f32((size_t)kGfCount * J);
    const std::vector<double>* src[kGfCount] = {&h, &ih, &lo, &up, &iden, &cp};
    for (int k = 0; k < kGfCount; ++k)
      for (int i = 0; i < J; ++i) f32[(size_t)k * J + i] = (float)(*src[k])[i];
    PES_CHECK_CUDA(cudaMemcpy(gf, f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice));
    std::vector<FF> fff((size_t)kGfCount * J);
    for (int k = 0; k < kGfCount; ++k)
      for (int i = 0; i < J; ++i) fff[(size_t)k * J + i] = ff_from((*src[k])[i]);
    PES_CHECK_CUDA(cudaMemcpy(gff, fff.data(), sizeof(FF) * fff.size(), cudaMemcpyHostToDevice));
  }
  PES_CHECK_CUDA(cudaMemcpy(chb, cb.data(), sizeof(int32_t) * M.nchunks, cudaMemcpyHostToDevice));
  PES_CHECK_CUDA(cudaMemcpy(chl, cl.data(), sizeof(int32_t) * M.nchunks, cudaMemcpyHostToDevice));
  PES_CHECK_CUDA(cudaMemcpy(chi, ci.data(), sizeof(int32_t) * M.nchunks, cudaMemcpyHostToDevice));
  PES_CHECK_CUDA(cudaMemcpy(bin_t, bt.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  PES_CHECK_CUDA(cudaMemset(pk, 0, sizeof(float4) * nd * 3 * n));
  PES_CHECK_CUDA(cudaMemset(ddv, 0, sizeof(float2) * nd * n));
  M.node_f = node_f;
  M.ch_begin = chb;
  M.ch_len = chl;
  M.ch_iv = chi;
  M.bin_t = bin_t;
  M.runs = runs;
  M.pk = pk;
  M.dd = ddv;
  M.nsp = nsp;
  M.vcut = vcut;
  M.pkink = nullptr;
  if (multi) {
    float4* pkink = nullptr;
    if ((rc = alloc(mb, &pkink, (size_t)V * 2))) return rc;
    M.pkink = pkink;
  }
  M.nch = nch;
  M.xbin = xbin;
  M.xbind = xbind;
  M.iv_first = ivfirst;
  M.xpart = xpart;
  M.xgpart = xgpart;
  M.gh = gh;
  M.ginvh = ginvh;
  M.glo = glo;
  M.gup = gup;
  M.ginvden = ginvden;
  M.gcp = gcp;
  M.gf = gf;
  M.gff = gff;
  M.tdn = tdn;
  M.tdn_ff = tdn_ff;
  M.sff = sff;
  M.cfrac = cfrac;
  M.node_ff = node_ff;
  M.yv = yv;
  M.scr = scr;
  M.cphi = cphi;
  M.cg = cg;
  M.mom = mom;
  M.ybar = ybar;
  M.part = part;
  M.gpart = gpart;
  M.gdir = gdir;
  M.gblocks = gblk;
  M.kinkR = kR;
  M.kinkC = kC;
  M.kinkF = kF;
  M.kinkM = kM;
  M.wmom = wmom;
  M.wtot = wtot;
  M.dsuf = dsuf;
  M.wrow = wrow;
  M.cgb = cgb;
  M.hd = hdv;
  M.ym = ymv;
  M.cbump = cbump;
  M.wspike = wspk;
  PES_CHECK_CUDA(cudaMemset(wspk, 0, sizeof(int32_t) * nd * J));
  M.rpart = rpart;
  M.rblocks = kRefineBlocks;
  M.refine_all = 0;
  M.rkind = rkind;
  M.fpart = fpart;
  M.xff = xff;
  {
    // the T channel's zeros f = n / L in the band (equal-arm constellations)
    std::vector<int32_t> zb((size_t)nd * kZeroMax, 0);
    int most = 0;
    for (int k = 0; k < PES_MAX_DETECTORS; ++k) M.nzb[k] = 0;
    for (int k = 0; k < nd; ++k) {
      std::vector<int32_t> bins;
      const double L = d.det[k].orbit.arm_sec;
      for (int zn = 1; L > 0.0 && zn / L <= fhi + kZeroHalf * d.f_step; ++zn) {
        const int64_t c = std::llround(zn / L / d.f_step) - d.k0;
        for (int64_t i = c - kZeroHalf; i <= c + kZeroHalf; ++i)
          if (i >= 0 && i < n) bins.push_back((int32_t)i);
      }
      std::sort(bins.begin(), bins.end());
      bins.erase(std::unique(bins.begin(), bins.end()), bins.end());
      PES_REQUIRE(bins.size() <= (size_t)kZeroMax,
                  "mixed plan: detector %d has %zu bins in T-channel zero windows (at most %d)", k, bins.size(),
                  kZeroMax);
      std::copy(bins.begin(), bins.end(), zb.begin() + (size_t)k * kZeroMax);
      M.nzb[k] = (int32_t)bins.size();
      most = std::max(most, M.nzb[k]);
    }
    int32_t* zbin = nullptr;
    double *zpart = nullptr, *zgpart = nullptr;
    M.zblocks = (int32_t)std::min<int64_t>(ceil_div(most, kExactThreads), 8);
    if ((rc = alloc(mb, &zbin, zb.size())) || (rc = alloc(mb, &zpart, (size_t)B * std::max(1, M.zblocks))) ||
        (rc = alloc(mb, &zgpart, (size_t)B * std::max(1, M.zblocks) * 11)))
      return rc;
    PES_CHECK_CUDA(cudaMemcpy(zbin, zb.data(), sizeof(int32_t) * zb.size(), cudaMemcpyHostToDevice));
    mb->zbin_host = zb;
    M.zbin = zbin;
    M.zgblocks = nullptr;
    if (M.zblocks > 0 && !multi) {
      SampleBlock<ZScalar>* zgb = nullptr;
      if ((rc = alloc(mb, &zgb, (size_t)B))) return rc;
      M.zgblocks = zgb;
    }
    M.zpart = zpart;
    M.zgpart = zgpart;
  }
  PES_CHECK_CUDA(cudaMemset(rkind, 0, sizeof(int32_t) * B));
  PES_CHECK_CUDA(cudaMemset(xff, 0, sizeof(float4) * nd * 6 * n));
  {
    // interval midpoints and their TDI delay factors (the last node has no interval)
    std::vector<float2> mff(J);
    std::vector<float4> tmf((size_t)nd * J);
    for (int jj = 0; jj < J; ++jj) {
      const double fm = jj + 1 < J ? 0.5 * (nf[jj] + nf[jj + 1]) : nf[jj];
      const FF v = ff_from(fm);
      mff[jj] = make_float2(v.hi, v.lo);
      for (int k = 0; k < nd; ++k) {
        Cx<double> D, Pf;
        tdi_factors(fm, d.det[k].orbit.arm_sec, d.det[k].generation == 20, D, Pf);
        const FF re = ff_from(D.re), im = ff_from(D.im);
        tmf[(size_t)k * J + jj] = make_float4(re.hi, re.lo, im.hi, im.lo);
      }
    }
    PES_CHECK_CUDA(cudaMemcpy(mid_ff, mff.data(), sizeof(float2) * J, cudaMemcpyHostToDevice));
    PES_CHECK_CUDA(cudaMemcpy(tdm_ff, tmf.data(), sizeof(float4) * tmf.size(), cudaMemcpyHostToDevice));
  }
  M.mid_ff = mid_ff;
  M.tdm_ff = tdm_ff;
  PES_CHECK_CUDA(cudaMemset(wmom, 0, sizeof(FF) * wn));
  PES_CHECK_CUDA(cudaMemset(wtot, 0, sizeof(FF) * wj));
  PES_CHECK_CUDA(cudaMemset(dsuf, 0, sizeof(double) * nd * (n + 1)));
  // the dense-path partial buffer is not needed; gradient set-up blocks are shared
  return PES_OK;
}

void mixed_stage_option(PesPlan* p, int set, int64_t* value) {
  if (set)
    p->mixed->stage_grad = *value != 0;
  else
    *value = p->mixed->stage_grad ? 1 : 0;
}

void mixed_refine_option(PesPlan* p, int set, int64_t* value) {
  if (set)
    p->mixed->dev.refine_all = *value != 0;
  else
    *value = p->mixed->dev.refine_all;
}

void mixed_destroy(PesPlan* p) {
  if (!p->mixed) return;
  if (p->mixed->side) cudaStreamSynchronize(p->mixed->side);
  if (p->mixed->aux) cudaStreamSynchronize(p->mixed->aux);
  for (cudaEvent_t e : {p->mixed->ev_nodes, p->mixed->ev_tfit, p->mixed->ev_dense, p->mixed->ev_tadj, p->mixed->ev_hd,
                        p->mixed->ev_pfit, p->mixed->ev_kink, p->mixed->ev_xgrad})
    if (e) cudaEventDestroy(e);
  if (p->mixed->aux) cudaStreamDestroy(p->mixed->aux);
  for (void* a : p->mixed->allocs) cudaFree(a);
  if (p->mixed->fork) cudaEventDestroy(p->mixed->fork);
  if (p->mixed->join) cudaEventDestroy(p->mixed->join);
  if (p->mixed->xready) cudaEventDestroy(p->mixed->xready);
  if (p->mixed->side) cudaStreamDestroy(p->mixed->side);
  delete p->mixed;
  p->mixed = nullptr;
}

}  // namespace pes

// Called from pes_plan_set_data with the caller's FP64 arrays.
namespace pes {
int mixed_ingest(PesPlan* p, int det, const double* data, const double* psd, cudaStream_t st) {
  MixedDev& M = p->mixed->dev;
  k_mixed_ingest<<<ceil_div(p->desc.nbins, 256), 256, 0, st>>>(p->dev, M, det,
                                                               reinterpret_cast<const double2*>(data), psd);
  PES_CHECK_LAUNCH();
  suffix_sum(p->desc.nbins, M.wrow, const_cast<double*>(M.dsuf) + (size_t)det * (p->desc.nbins + 1), st);
  PES_CHECK_LAUNCH();
  k_wmoments<<<ceil_div((M.J - 1) * 3, 128), 128, 0, st>>>(p->dev, M, det, const_cast<FF*>(M.wmom),
                                                            const_cast<FF*>(M.wtot));
  PES_CHECK_LAUNCH();
  k_wspike<<<ceil_div(M.J, 128), 128, 0, st>>>(p->dev, M, det, const_cast<int32_t*>(M.wspike));
  PES_CHECK_LAUNCH();
  return PES_OK;
}

// Dense model of every detector for one parameter set: out (n_det, 3, nbins) complex.
int mixed_model(PesPlan* p, const double* theta_dev, double* out, cudaStream_t st) {
  MixedDev& M = p->mixed->dev;
  const GenArg& G = p->mixed->gen;
  SampleBlock<double>* blocks = reinterpret_cast<SampleBlock<double>*>(p->blocks);
  k_setup<double><<<1, 64, 0, st>>>(p->dev, theta_dev, 1, 0, blocks, hm_blocks<double>(p));
  PES_CHECK_LAUNCH();
  const unsigned nm = (unsigned)M.n_modes;
  k_mixed_ranges<0><<<1, 64, 0, st>>>(p->dev, M, blocks, 1);
  k_mixed_ranges<1><<<1, 64, 0, st>>>(p->dev, M, blocks, 1);
  PES_CHECK_LAUNCH();
  k_kink<<<1, 64, 0, st>>>(p->dev, M, G, blocks, 1);
  PES_CHECK_LAUNCH();
  k_sparse_fwd<false><<<dim3(M.nblk_sparse, M.n_det, nm), kSparseThreads, 0, st>>>(p->dev, M, G, blocks);
  PES_CHECK_LAUNCH();
  launch_spline_fit(M, nm, st, st);
  PES_CHECK_LAUNCH();
  k_sparse_fwd<true><<<dim3(M.nblk_sparse, M.n_det, nm), kSparseThreads, 0, st>>>(p->dev, M, G, blocks);
  k_bump<<<(unsigned)ceil_div(nm * M.n_det * (int64_t)M.J, (int64_t)128), 128, 0, st>>>(M, blocks, 1);
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * M.n_det * 3 * p->desc.nbins, st));
  k_run_anchors<<<dim3((unsigned)ceil_div(M.nchunks, 128), M.n_det, nm), 128, 0, st>>>(p->dev, M, blocks);
  PES_CHECK_LAUNCH();
  if (nm > 1)
    k_dense_mixed<2, false, kHMModes><<<dim3(M.nblk_dense, 1), kMixThreads, 0, st>>>(
        p->dev, M, blocks, reinterpret_cast<double2*>(out));
  else
    k_dense_mixed<2, false, 1><<<dim3(M.nblk_dense, 1), kMixThreads, 0, st>>>(p->dev, M, blocks,
                                                                     reinterpret_cast<double2*>(out));
  PES_CHECK_LAUNCH();
  k_exact<2, double><<<dim3(M.xblocks, 1), kExactThreads, 0, st>>>(p->dev, M, G, blocks,
                                                                      reinterpret_cast<double2*>(out));
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int mixed_work(PesPlan* p, int64_t B, const std::vector<int64_t>& kcut, const std::vector<int32_t>& ok,
               int64_t* out, cudaStream_t st) {
  const MixedDev& M = p->mixed->dev;
  const int nm = M.n_modes;
  std::vector<int32_t> xb((size_t)B * nm * M.n_det), ns((size_t)B * nm), rk((size_t)B);
  if (B > 0) {
    PES_CHECK_CUDA(cudaMemcpy(xb.data(), M.xbind, sizeof(int32_t) * xb.size(), cudaMemcpyDeviceToHost));
    PES_CHECK_CUDA(cudaMemcpy(ns.data(), M.nsp, sizeof(int32_t) * ns.size(), cudaMemcpyDeviceToHost));
    PES_CHECK_CUDA(cudaMemcpy(rk.data(), M.rkind, sizeof(int32_t) * rk.size(), cudaMemcpyDeviceToHost));
  }
  // dense and exact bins per sample (a bin sums all modes); sparse nodes per mode
  for (int64_t s = 0; s < B; ++s) {
    if (!ok[s]) continue;
    for (int d = 0; d < M.n_det; ++d) {
      const int64_t x = xb[(size_t)s * nm * M.n_det + d];
      int64_t zw = 0;  // window bins in [x, kcut): exact, not through the dense stage
      for (int t = 0; t < M.nzb[d]; ++t) {
        const int32_t i = p->mixed->zbin_host[(size_t)d * kZeroMax + t];
        zw += i >= x && i < kcut[s];
      }
      out[0] += kcut[s] - x - zw;
      out[1] += x + zw;
    }
    for (int k = 0; k < nm; ++k)
      if (ns[(size_t)s * nm + k] >= 3) out[2] += (int64_t)(ns[(size_t)s * nm + k] + 1) * M.n_det;
    out[4] += rk[s] == kRefineFF;
    out[5] += rk[s] == kRefineExact;
  }
  (void)st;
  return PES_OK;
}

int mixed_lnl(PesPlan* p, const double* theta, int64_t B, double* lnl, double* grad, int32_t* status,
              cudaStream_t st) {
  MixedDev& M = p->mixed->dev;
  const GenArg& G = p->mixed->gen;
  SampleBlock<double>* blocks = reinterpret_cast<SampleBlock<double>*>(p->blocks);
  const bool multi = M.n_modes > 1;
  const int64_t V = B * M.n_modes;  // virtual samples (sample, mode)
  PES_REQUIRE(!(grad && multi), "mixed plan: the gradient is implemented for IMRPhenomD plans only "
                                "(the FP64 plan gives IMRPhenomHM gradients)");
  {
    ProfScope ps(p, kKSetup, st);
    k_setup<double><<<ceil_div(B, p->sample_threads), p->sample_threads, 0, st>>>(p->dev, theta, B, 0, blocks,
                                                                                  hm_blocks<double>(p));
  }
  PES_CHECK_LAUNCH();
  {
    ProfScope ps(p, kKOther, st);
    k_mixed_ranges<0><<<ceil_div(V, 64), 64, 0, st>>>(p->dev, M, blocks, B);
  }
  PES_CHECK_LAUNCH();
  // side stream: the exact-bin range, the exact bins and the gradient set-up they need
  cudaStream_t side = p->mixed->side;
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->fork, st));
  PES_CHECK_CUDA(cudaStreamWaitEvent(side, p->mixed->fork, 0));
  {
    ProfScope ps(p, kKOther, side);
    k_mixed_ranges<1><<<ceil_div(B, p->sample_threads), p->sample_threads, 0, side>>>(p->dev, M, blocks, B);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->xready, side));
  {
    ProfScope ps(p, kKDenseFp64, side);
    k_exact<0, double><<<dim3(M.xblocks, (unsigned)B), kExactThreads, 0, side>>>(p->dev, M, G, blocks, nullptr);
  }
  PES_CHECK_LAUNCH();
  if (M.zblocks > 0) {
    ProfScope ps(p, kKDenseFp64, side);
    k_exact<4, double><<<dim3(M.zblocks, (unsigned)B), kExactThreads, 0, side>>>(p->dev, M, G, blocks, nullptr);
  }
  PES_CHECK_LAUNCH();
  if (grad) {
    {
      ProfScope ps(p, kKSetup, side);
      k_setup_grad<<<ceil_div(B, p->sample_threads), p->sample_threads, 0, side>>>(p->dev, theta, B,
                                                     reinterpret_cast<SampleBlock<GradScalar>*>(M.gblocks));
    }
    PES_CHECK_LAUNCH();
    {
      ProfScope ps(p, kKDenseFp64, side);
      k_exact<1, GradScalar><<<dim3(M.xblocks, (unsigned)B), kExactThreads, 0, side>>>(
          p->dev, M, G, reinterpret_cast<const SampleBlock<GradScalar>*>(M.gblocks), nullptr);
    }
    PES_CHECK_LAUNCH();
    if (M.zblocks > 0) {
      ProfScope ps(p, kKDenseFp64, side);
      SampleBlock<ZScalar>* zb = reinterpret_cast<SampleBlock<ZScalar>*>(M.zgblocks);
      k_setup<ZScalar><<<ceil_div(B, p->sample_threads), p->sample_threads, 0, side>>>(p->dev, theta, B, 0, zb,
                                                                                       nullptr);
      k_zero_grad<<<dim3(M.zblocks, (unsigned)B), kExactThreads, 0, side>>>(p->dev, M, zb);
    }
    PES_CHECK_LAUNCH();
    // the backward node stage reads the gradient set-up
    PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_xgrad, side));
  }
  // (the side stream's completion is recorded after the exact re-evaluation below)
  {
    ProfScope ps(p, kKSparse, st);
    k_kink<<<ceil_div(V * M.n_det, p->sample_threads), p->sample_threads, 0, st>>>(p->dev, M, G, blocks, B);
  }
  PES_CHECK_LAUNCH();
  cudaStream_t aux = p->mixed->aux;
  {
    // the exact model at the interval midpoints, beside the node values
    PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_kink, st));
    PES_CHECK_CUDA(cudaStreamWaitEvent(aux, p->mixed->ev_kink, 0));
    ProfScope ps(p, kKSparse, aux);
    k_sparse_fwd<true><<<dim3(M.nblk_sparse, M.n_det, (unsigned)V), kSparseThreads, 0, aux>>>(p->dev, M, G, blocks);
  }
  PES_CHECK_LAUNCH();
  {
    ProfScope ps(p, kKSparse, st);
    dim3 grid(M.nblk_sparse, M.n_det, (unsigned)V);
    k_sparse_fwd<false><<<grid, kSparseThreads, 0, st>>>(p->dev, M, G, blocks);
  }
  PES_CHECK_LAUNCH();
  {
    // the phase fit here, the transfer fit on the second stream
    PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_nodes, st));
    PES_CHECK_CUDA(cudaStreamWaitEvent(aux, p->mixed->ev_nodes, 0));
    ProfScope ps(p, kKSpline, st);
    ProfScope ps_aux(p, kKSpline, aux);
    launch_spline_fit(M, V, st, aux);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_pfit, st));
  {
    // the midpoint corrections, after both fits (grids beyond 64 x 32 intervals
    // fit every quantity on the main stream)
    PES_CHECK_CUDA(cudaStreamWaitEvent(aux, p->mixed->ev_pfit, 0));
    ProfScope ps(p, kKSpline, aux);
    k_bump<<<(unsigned)ceil_div(V * M.n_det * (int64_t)M.J, (int64_t)128), 128, 0, aux>>>(M, blocks, B);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_tfit, aux));
  {
    // <h|h> and <d|d> of the dense ranges (per mode), beside the anchors and the dense stage
    PES_CHECK_CUDA(cudaStreamWaitEvent(aux, p->mixed->xready, 0));
    ProfScope ps(p, kKOther, aux);
    k_hd<<<(unsigned)(V * M.n_det), kHdThreads, 0, aux>>>(p->dev, M, blocks, B);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_hd, p->mixed->aux));
  // After the dense stage (its rounding sums) and k_hd: which samples to
  // re-evaluate and how, then the re-evaluations, on the side stream after
  // its exact low-frequency bins (beside the adjoint stages of lnL+gradient
  // calls, where they do not take SMs from the dense stage).
  auto refine = [&]() -> int {
    PES_CHECK_CUDA(cudaStreamWaitEvent(side, p->mixed->ev_dense, 0));
    {
      ProfScope ps(p, kKOther, side);
      k_refine_select<<<ceil_div(B, 64), 64, 0, side>>>(p->dev, M, blocks, B);
    }
    PES_CHECK_LAUNCH();
    {
      ProfScope ps(p, kKDenseFp64, side);
      k_exact<3, double><<<dim3(M.rblocks, (unsigned)B), kExactThreads, 0, side>>>(p->dev, M, G, blocks, nullptr);
    }
    PES_CHECK_LAUNCH();
    {
      ProfScope ps(p, kKOther, side);
      if (multi)
        k_dense_ff<kHMModes><<<dim3(M.nblk_dense, (unsigned)B), kMixThreads, 0, side>>>(p->dev, M, blocks);
      else
        k_dense_ff<1><<<dim3(M.nblk_dense, (unsigned)B), kMixThreads, 0, side>>>(p->dev, M, blocks);
    }
    PES_CHECK_LAUNCH();
    PES_CHECK_CUDA(cudaEventRecord(p->mixed->join, side));
    return PES_OK;
  };
  PES_CHECK_CUDA(cudaStreamWaitEvent(side, p->mixed->ev_hd, 0));
  if (grad) {
    PES_CHECK_CUDA(cudaMemsetAsync(M.mom, 0, sizeof(float) * B * M.n_det * M.J * kNodeQ * kMoments, st));
    PES_CHECK_CUDA(cudaMemsetAsync(M.kinkM, 0, sizeof(float) * B * M.n_det * 12, st));
  }
  PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->xready, 0));
  {
    ProfScope ps(p, kKSpline, st);
    dim3 grid((unsigned)ceil_div(M.nchunks, 128), M.n_det, (unsigned)V);
    k_run_anchors<<<grid, 128, 0, st>>>(p->dev, M, blocks);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->ev_tfit, 0));
  {
    ProfScope ps(p, kKDenseMixed, st);
    dim3 grid(M.nblk_dense, (unsigned)B);
    if (grad)
      if (p->mixed->stage_grad)
        k_dense_mixed<1, true, 1><<<grid, kMixThreads, 0, st>>>(p->dev, M, blocks, nullptr);
      else
        k_dense_mixed<1, false, 1><<<grid, kMixThreads, 0, st>>>(p->dev, M, blocks, nullptr);
    else if (multi)
      k_dense_mixed<0, false, kHMModes><<<grid, kMixThreads, 0, st>>>(p->dev, M, blocks, nullptr);
    else
      k_dense_mixed<0, true, 1><<<grid, kMixThreads, 0, st>>>(p->dev, M, blocks, nullptr);
  }
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_dense, st));
  if (!grad) {
    const int rc = refine();
    if (rc != PES_OK) return rc;
  }
  auto finalize = [&]() -> int {
    PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->join, 0));
    PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->ev_hd, 0));
    {
      ProfScope ps(p, kKFinalize, st);
      k_mixed_finalize<<<ceil_div(B, 64), 64, 0, st>>>(p->dev, M, blocks, B, lnl, status);
    }
    PES_CHECK_LAUNCH();
    return PES_OK;
  };
  if (!grad) return finalize();
  {
    const int rc = refine();
    if (rc != PES_OK) return rc;
  }
  // node adjoints: phase systems here, transfer systems on the second stream;
  // then the backward node stage
  const double ws = 4.0 * p->dev.df;
  const dim3 sgrid(M.nblk_sparse, M.n_det, (unsigned)B);
  if (spline_seg(M.J) == 32) {
    const int64_t nsd = B * M.n_det;
    {
      ProfScope ps(p, kKAdjoint, st);
      k_spline_adjoint_staged<double><<<(unsigned)ceil_div(nsd, (int64_t)kFitWarps), kFitWarps * 32,
                                        adj_smem_bytes<double>(M.J), st>>>(M, nsd, ws);
    }
    PES_CHECK_LAUNCH();
    PES_CHECK_CUDA(cudaStreamWaitEvent(aux, p->mixed->ev_dense, 0));
    {
      ProfScope ps(p, kKAdjoint, aux);
      k_spline_adjoint_staged<float><<<(unsigned)ceil_div(nsd * 6, (int64_t)kFitWarps), kFitWarps * 32,
                                       adj_smem_bytes<float>(M.J), aux>>>(M, nsd * 6, ws);
    }
    PES_CHECK_LAUNCH();
  } else {
    ProfScope ps(p, kKAdjoint, st);
    if (spline_seg(M.J) == kSegMax)
      k_spline_adjoint<kSegMax><<<(unsigned)(B * M.n_det * kNodeQ), 32, 0, st>>>(M, ws);
    else
      k_spline_adjoint_wide<<<(unsigned)(B * M.n_det), kSplineThreads, 0, st>>>(M, ws);
    PES_CHECK_LAUNCH();
  }
  PES_CHECK_CUDA(cudaEventRecord(p->mixed->ev_tadj, aux));
  PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->ev_tadj, 0));
  PES_CHECK_CUDA(cudaStreamWaitEvent(st, p->mixed->ev_xgrad, 0));
  {
    ProfScope ps(p, kKAdjoint, st);
    k_sparse_bwd_split<<<sgrid, kSparseThreads, 0, st>>>(p->dev, M, G, ws);
  }
  PES_CHECK_LAUNCH();
  {
    // the lnL sums, after the side stream's exact passes (exact-bin gradient
    // partials, refined samples), then the gradient sums
    const int rc = finalize();
    if (rc != PES_OK) return rc;
  }
  {
    ProfScope ps(p, kKFinalize, st);
    k_mixed_grad_finalize<<<ceil_div(B, 64), 64, 0, st>>>(M, B, -2.0 * p->dev.df, grad);
  }
  PES_CHECK_LAUNCH();
  return PES_OK;
}

}  // namespace pes
