// Per-frequency physics of the FD response path, templated on the scalar type
// (double, or Dual<N> for exact parameter derivatives):
//   * Keplerian constellation orbits   pespace/detector/orbit.py:260-322, 362-419
//   * polarisation tensors, k          pespace/detector/antenna.py:42-114
//   * six single-link responses        pespace/detector/antenna.py:429-543
//   * TDI X/Y/Z -> A/E/T               pespace/detector/tdi.py:1683-1793
//   * IMRPhenomD (2,2) amplitude, phase and t(f) (Husa et al. 2016,
//     arXiv:1508.07250; Khan et al. 2016, arXiv:1508.07253), evaluated from a
//     per-sample coefficient block as polynomials in u = (M f)^{1/3}.
#pragma once

#include "pes_common.cuh"
#include "pes_ff.cuh"
#include "../../include/pespace_gb300.h"

namespace pes {

// ------------------------------------------------------------------ orbits
// An orbit's parameters as float-float values (same field names as PesOrbit),
// for node evaluations in FF arithmetic.
struct OrbitFF {
  int32_t kind;
  int32_t pad;
  FF arm_sec, rotation_initial, revolution_initial, omega_revolution, r_sec, omega_rotation;
  FF slam_ref, clam_ref, sbeta_ref, cbeta_ref;
  FF ck[3], sk[3];
};

// The same in FP32, for derivative passes that run entirely on the FP32 pipes.
struct OrbitF {
  int32_t kind;
  int32_t pad;
  float arm_sec, rotation_initial, revolution_initial, omega_revolution, r_sec, omega_rotation;
  float slam_ref, clam_ref, sbeta_ref, cbeta_ref;
  float ck[3], sk[3];
};

PES_HD OrbitF orbit_f(const PesOrbit& o) {
  OrbitF r;
  r.kind = o.kind;
  r.pad = 0;
  r.arm_sec = (float)o.arm_sec;
  r.rotation_initial = (float)o.rotation_initial;
  r.revolution_initial = (float)o.revolution_initial;
  r.omega_revolution = (float)o.omega_revolution;
  r.r_sec = (float)o.r_sec;
  r.omega_rotation = (float)o.omega_rotation;
  r.slam_ref = (float)o.slam_ref;
  r.clam_ref = (float)o.clam_ref;
  r.sbeta_ref = (float)o.sbeta_ref;
  r.cbeta_ref = (float)o.cbeta_ref;
  for (int k = 0; k < 3; ++k) {
    r.ck[k] = (float)o.ck[k];
    r.sk[k] = (float)o.sk[k];
  }
  return r;
}

inline OrbitFF orbit_ff(const PesOrbit& o) {
  OrbitFF r;
  r.kind = o.kind;
  r.pad = 0;
  r.arm_sec = ff_from(o.arm_sec);
  r.rotation_initial = ff_from(o.rotation_initial);
  r.revolution_initial = ff_from(o.revolution_initial);
  r.omega_revolution = ff_from(o.omega_revolution);
  r.r_sec = ff_from(o.r_sec);
  r.omega_rotation = ff_from(o.omega_rotation);
  r.slam_ref = ff_from(o.slam_ref);
  r.clam_ref = ff_from(o.clam_ref);
  r.sbeta_ref = ff_from(o.sbeta_ref);
  r.cbeta_ref = ff_from(o.cbeta_ref);
  for (int k = 0; k < 3; ++k) {
    r.ck[k] = ff_from(o.ck[k]);
    r.sk[k] = ff_from(o.sk[k]);
  }
  return r;
}

// n[i] = unit vector of link i+1 (n1: 2->3, n2: 3->1, n3: 1->2); xd[i] = node
// i+1 relative to the constellation centre x0 (light-seconds, SSB axes).
template <class T, class O>
PES_HD void constellation_parts(const O& o, const T& t, T n[3][3], T xd[3][3], T x0[3]) {
  T c0, s0;
  T alpha = o.omega_revolution * t + o.revolution_initial;
  dsincos(alpha, &s0, &c0);
  if (o.kind == 0) {
    // x_k,det = r' (sa ca sk - (1+sa^2) ck, sa ca ck - (1+ca^2) sk, -sqrt3 (ca ck + sa sk))
    const T sc = s0 * c0, s2 = s0 * s0, c2 = c0 * c0;
    const double sqrt3 = 1.7320508075688772;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xd[k][0] = o.r_sec * (sc * o.sk[k] - (1.0 + s2) * o.ck[k]);
      xd[k][1] = o.r_sec * (sc * o.ck[k] - (1.0 + c2) * o.sk[k]);
      xd[k][2] = o.r_sec * (-sqrt3 * (c0 * o.ck[k] + s0 * o.sk[k]));
    }
  } else {
    // node phases kappa_k = kappa_1 + 2 pi (k-1)/3, by angle addition
    T kap = o.omega_rotation * t + o.rotation_initial;
    T sk1, ck1;
    dsincos(kap, &sk1, &ck1);
    const double c3 = -0.5, s3 = 0.86602540378443865;  // cos, sin of 2pi/3
    T cks[3], sks[3];
    cks[0] = ck1;
    sks[0] = sk1;
    cks[1] = ck1 * c3 - sk1 * s3;
    sks[1] = sk1 * c3 + ck1 * s3;
    cks[2] = ck1 * c3 + sk1 * s3;
    sks[2] = sk1 * c3 - ck1 * s3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xd[k][0] = o.r_sec * (o.sbeta_ref * o.clam_ref * sks[k] + o.slam_ref * cks[k]);
      xd[k][1] = o.r_sec * (o.sbeta_ref * o.slam_ref * sks[k] - o.clam_ref * cks[k]);
      xd[k][2] = o.r_sec * (-o.cbeta_ref * sks[k]);
    }
  }
  const auto inv_arm = lift<decltype(o.arm_sec)>(1.0) / o.arm_sec;
  x0[0] = c0 * kAUsec;
  x0[1] = s0 * kAUsec;
  x0[2] = lift<T>(0.0);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    n[0][j] = (xd[2][j] - xd[1][j]) * inv_arm;
    n[1][j] = (xd[0][j] - xd[2][j]) * inv_arm;
    n[2][j] = (xd[1][j] - xd[0][j]) * inv_arm;
  }
}

// Node positions in the SSB frame: x = xd + x0.
template <class T>
PES_HD void constellation(const PesOrbit& o, const T& t, T n[3][3], T x[3][3]) {
  T xd[3][3], x0[3];
  constellation_parts(o, t, n, xd, x0);
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) x[k][j] = xd[k][j] + x0[j];
}

// e+ = p p - q q, ex = p q + q p (symmetric: 6 independent entries each), k.
template <class T>
struct Polar {
  T P[6], X[6];  // xx, xy, xz, yy, yz, zz
  T k[3];
};

template <class T>
PES_HD void make_polar(const T& lam, const T& sb, const T& cb, const T& psi, Polar<T>& o) {
  T sl, cl, sp, cp;
  dsincos(lam, &sl, &cl);
  dsincos(psi, &sp, &cp);
  T p[3] = {sl * cp - cl * sb * sp, -cl * cp - sl * sb * sp, cb * sp};
  T q[3] = {-sl * sp - cl * sb * cp, cl * sp - sl * sb * cp, cb * cp};
  const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    o.P[m] = p[ii[m]] * p[jj[m]] - q[ii[m]] * q[jj[m]];
    o.X[m] = p[ii[m]] * q[jj[m]] + q[ii[m]] * p[jj[m]];
  }
  o.k[0] = -(cb * cl);
  o.k[1] = -(cb * sl);
  o.k[2] = -sb;
}

// n^T M n for a symmetric M stored as 6 entries
template <class T>
PES_HD T quad6(const T n[3], const T M[6]) {
  return n[0] * n[0] * M[0] + n[1] * n[1] * M[3] + n[2] * n[2] * M[5] +
         2.0 * (n[0] * n[1] * M[1] + n[0] * n[2] * M[2] + n[1] * n[2] * M[4]);
}

template <class T>
PES_HD T sinc_ref(const T& x) {
  // utils.py:60-79: sin(x)/x with the x == 0 guard
  return (x.v == 0) ? lift<T>(1.0) : dsin(x) / x;
}
PES_HD FF sinc_ref(const FF& x) { return ff_sinc(x); }
// FF value, FP32 tangents: d/dx sin(x)/x = x sum_k (-1)^k 2k x^(2k-2) / (2k+1)!
// (k = 1..8, truncation below 2e-9 relative for |x| <= 2), (cos x - sinc x) / x beyond.
template <int N, class D>
PES_HD Dual<N, D, FF> sinc_ref(const Dual<N, D, FF>& x) {
  Dual<N, D, FF> r;
  r.v = ff_sinc(x.v);
  const float xf = x.v.hi;
  float ds;
  if (fabsf(xf) <= 2.0f) {
    const float z = xf * xf;
    float p = 1.0f / 22230464256000.0f;
    p = fmaf(p, z, -1.0f / 93405312000.0f);
    p = fmaf(p, z, 1.0f / 518918400.0f);
    p = fmaf(p, z, -1.0f / 3991680.0f);
    p = fmaf(p, z, 1.0f / 45360.0f);
    p = fmaf(p, z, -1.0f / 840.0f);
    p = fmaf(p, z, 1.0f / 30.0f);
    p = fmaf(p, z, -1.0f / 3.0f);
    ds = p * xf;
  } else {
    FF sn, cs;
    dsincos(x.v, &sn, &cs);
    ds = (cs.hi - r.v.hi) / xf;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * D(ds);
  return r;
}
PES_HD double sinc_ref(const double& x) {
  if (::fabs(x) <= 2.0) {
    double s, ds;
    sinc_taylor(x, &s, &ds);
    return s;
  }
  return ::sin(x) / x;
}
template <int N, class D>
PES_HD Dual<N, D, double> sinc_ref(const Dual<N, D, double>& x) {
  if (::fabs(x.v) <= 2.0) {
    double s, ds;
    sinc_taylor(x.v, &s, &ds);
    return chain1(x, s, ds);
  }
  return dsin(x) / x;
}

// Six single-link responses of one time-shifted mode (hp, hc at f; tf already
// includes t_c).  Order: 12, 21, 23, 32, 31, 13.  With kFactorDoppler the
// propagation delays use node positions relative to the constellation centre
// and the centre's delay k.x0 is returned instead (the links then miss the
// factor exp(-2 pi i f k.x0)); otherwise the links are those of antenna.py.
template <bool kFactorDoppler, class T, class O, class Fq>
PES_HD void single_links_impl(const O& o, Fq f, const Cx<T>& hp, const Cx<T>& hc, const T& tf,
                              const Polar<T>& pol, Cx<T> out[6], T* kx0_out) {
  T n[3][3], xd[3][3], x0[3];
  constellation_parts(o, tf, n, xd, x0);
  Cx<T> nh[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T fp = quad6(n[i], pol.P), fc = quad6(n[i], pol.X);
    nh[i] = cscale(fp, hp) + cscale(fc, hc);
  }
  T kn[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) kn[i] = pol.k[0] * n[i][0] + pol.k[1] * n[i][1] + pol.k[2] * n[i][2];
  T kx[3];  // k.(x1+x2), k.(x2+x3), k.(x3+x1)  (or with xd when factoring)
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int a = i, b = (i + 1) % 3;
    if (kFactorDoppler) {
      kx[i] = pol.k[0] * (xd[a][0] + xd[b][0]) + pol.k[1] * (xd[a][1] + xd[b][1]) + pol.k[2] * (xd[a][2] + xd[b][2]);
    } else {
      kx[i] = pol.k[0] * ((xd[a][0] + x0[0]) + (xd[b][0] + x0[0])) +
              pol.k[1] * ((xd[a][1] + x0[1]) + (xd[b][1] + x0[1])) +
              pol.k[2] * ((xd[a][2] + x0[2]) + (xd[b][2] + x0[2]));
    }
  }
  if (kFactorDoppler) *kx0_out = pol.k[0] * x0[0] + pol.k[1] * x0[1];
  const auto arm = o.arm_sec;
  const auto pifL = lift<Fq>(kPi) * f * arm;
  const auto ce = -(lift<Fq>(kPi) * f);
  Cx<T> e[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T a = ce * (arm + kx[i]);
    dsincos(a, &e[i].im, &e[i].re);
  }
  // prefactor -i pi f L:  (-i pifL) * nh = (pifL nh.im, -pifL nh.re)
  // link pairs: (12, 21) use n3 and e12; (23, 32) n1 and e23; (31, 13) n2 and e31
  const int nidx[3] = {2, 0, 1};
#pragma unroll
  for (int pr = 0; pr < 3; ++pr) {
    const int ni = nidx[pr];
    Cx<T> pre = cx(pifL * nh[ni].im, -(pifL * nh[ni].re));
    Cx<T> b = cmul(pre, e[pr]);
    T sp = sinc_ref(pifL * (1.0 + kn[ni]));
    T sm = sinc_ref(pifL * (1.0 - kn[ni]));
    out[2 * pr] = cscale(sp, b);
    out[2 * pr + 1] = cscale(sm, b);
  }
}

template <class T>
PES_HD void single_links(const PesOrbit& o, double f, const Cx<T>& hp, const Cx<T>& hc, const T& tf,
                         const Polar<T>& pol, Cx<T> out[6]) {
  single_links_impl<false, T>(o, f, hp, hc, tf, pol, out, nullptr);
}

// TDI delay factor D = exp(-2 pi i f L) and generation prefactor.
PES_HD void tdi_factors(double f, double arm, int gen20, Cx<double>& D, Cx<double>& P) {
  double s = -2.0 * kPi * f * arm;
  dsincos(s, &D.im, &D.re);
  Cx<double> D2 = cmul(D, D);
  if (!gen20) {
    P = cx(1.0 - D2.re, -D2.im);
  } else {
    Cx<double> D4 = cmul(D2, D2);
    Cx<double> D6 = cmul(D2, D4);
    P = cx(1.0 - D2.re - D4.re + D6.re, -D2.im - D4.im + D6.im);
  }
}

// X/Y/Z (or A/E/T) from the six links with delay factor Dt; kPre applies the
// generation prefactor Pt, else it is taken as 1.
template <bool kPre, class T>
PES_HD void tdi_channels_t(const Cx<T>& Dt, const Cx<T>& Pt, int orth, const Cx<T> L[6], Cx<T> out[3]) {
  // L: 0=12 1=21 2=23 3=32 4=31 5=13
  Cx<T> X = (L[5] - L[0]) + cmul(Dt, L[4] - L[1]);
  Cx<T> Y = (L[1] - L[2]) + cmul(Dt, L[0] - L[3]);
  Cx<T> Z = (L[3] - L[4]) + cmul(Dt, L[2] - L[5]);
  if (kPre) {
    X = cmul(Pt, X);
    Y = cmul(Pt, Y);
    Z = cmul(Pt, Z);
  }
  if (orth) {
    const double r2 = 0.70710678118654752, r6 = 0.40824829046386302, r3 = 0.57735026918962576;
    out[0] = cscale(r2, Z - X);
    out[1] = cx((X.re - 2.0 * Y.re + Z.re) * r6, (X.im - 2.0 * Y.im + Z.im) * r6);
    out[2] = cscale(r3, (X + Y) + Z);
  } else {
    out[0] = X;
    out[1] = Y;
    out[2] = Z;
  }
}

template <class T>
PES_HD void tdi_channels(const Cx<double>& D, const Cx<double>& P, int orth, const Cx<T> L[6], Cx<T> out[3]) {
  tdi_channels_t<true, T>(cx(lift<T>(D.re), lift<T>(D.im)), cx(lift<T>(P.re), lift<T>(P.im)), orth, L, out);
}

// ------------------------------------------------------------------ Kerr quasi-normal modes
// M omega = wR - i wI of a Kerr black hole of dimensionless spin a for mode
// `mode` (table order (2,2), (2,1), (3,3), (3,2), (4,4), (4,3); s = -2,
// overtone 0), from the natural cubic spline in u = sqrt(1 - a) through the
// frequencies that gen_qnm_table.py computes by Leaver's continued fractions
// (negative a: the retrograde continuation).  a is clamped to +-PES_QNM_A_MAX.
#define PES_QNM_STORAGE __device__ static const
#include "pes_qnm_table.h"

template <class T>
PES_HD void qnm_interp(int mode, const T& a, T& wR, T& wI) {
  T ac = a;
  if (val(ac) > PES_QNM_A_MAX) ac = lift<T>(PES_QNM_A_MAX);
  if (val(ac) < -PES_QNM_A_MAX) ac = lift<T>(-PES_QNM_A_MAX);
  const T u = dsqrt(1.0 - ac);
  int i = (int)floor((val(u) - PES_QNM_U0) / PES_QNM_DU);
  i = i < 0 ? 0 : (i > PES_QNM_NODES - 2 ? PES_QNM_NODES - 2 : i);
  const double h = PES_QNM_DU;
  const T t = (u - (PES_QNM_U0 + i * h)) / h;
  const T s = 1.0 - t;
  const T cA = (s * s * s - s) * (h * h / 6.0), cB = (t * t * t - t) * (h * h / 6.0);
  const double* re = kQnmTable[mode][0];
  const double* re2 = kQnmTable[mode][1];
  const double* im = kQnmTable[mode][2];
  const double* im2 = kQnmTable[mode][3];
  wR = s * re[i] + t * re[i + 1] + cA * re2[i] + cB * re2[i + 1];
  wI = s * im[i] + t * im[i + 1] + cA * im2[i] + cB * im2[i + 1];
}

// ------------------------------------------------------------------ IMRPhenomD
constexpr double kAmpJoinIns = 0.014;  // Mf of the inspiral/intermediate amplitude join
constexpr double kPhiJoinIns = 0.018;  // Mf of the inspiral/intermediate phase join
constexpr double kMfCut = 0.2;         // PhenomD is zero above Mf = 0.2

// Coefficient fits (Khan et al. 2016 Table V): v2, gamma1..3, sigma1..4, beta1..3, alpha1..5,
// rho1..3; value = c0 + c1 eta + xi (c2 + c3 eta + c4 eta^2) + xi^2 (c5 + ...) + xi^3 (c8 + ...),
// xi = chi_PN - 1.
enum { kFV2, kFG1, kFG2, kFG3, kFS1, kFS2, kFS3, kFS4, kFB1, kFB2, kFB3, kFA1, kFA2, kFA3, kFA4, kFA5,
       kFR1, kFR2, kFR3, kFCount };
__device__ __constant__ static const double kPhenomFits[kFCount][11] = {
  {0.8149838730507785, 2.5747553517454658, 1.1610198035496786, -2.3627771785551537, 6.771038707057573, 0.7570782938606834, -2.7256896890432474, 7.1140380397149965, 0.1766934149293479, -0.7978690983168183, 2.1162391502005153},
  {0.006927402739328343, 0.03020474290328911, 0.006308024337706171, -0.12074130661131138, 0.26271598905781324, 0.0034151773647198794, -0.10779338611188374, 0.27098966966891747, 0.0007374185938559283, -0.02749621038376281, 0.0733150789135702},
  {1.010344404799477, 0.0008993122007234548, 0.283949116804459, -4.049752962958005, 13.207828172665366, 0.10396278486805426, -7.025059158961947, 24.784892370130475, 0.03093202475605892, -2.6924023896851663, 9.609374464684983},
  {1.3081615607036106, -0.005537729694807678, -0.06782917938621007, -0.6689834970767117, 3.403147966134083, -0.05296577374411866, -0.9923793203111362, 4.820681208409587, -0.006134139870393713, -0.38429253308696365, 1.7561754421985984},
  {2096.551999295543, 1463.7493168261553, 1312.5493286098522, 18307.330017082117, -43534.1440746107, -833.2889543511114, 32047.31997183187, -108609.45037520859, 452.25136398112204, 8353.439546391714, -44531.3250037322},
  {-10114.056472621156, -44631.01109458185, -6541.308761668722, -266959.23419307504, 686328.3229317984, 3405.6372187679685, -437507.7208209015, 1.6318171307344697e6, -7462.648563007646, -114585.25177153319, 674402.4689098676},
  {22933.658273436497, 230960.00814979506, 14961.083974183695, 1.1940181342318142e6, -3.1042239693052764e6, -3038.166617199259, 1.8720322849093592e6, -7.309145012085539e6, 42738.22871475411, 467502.018616601, -3.064853498512499e6},
  {-14621.71522218357, -377812.8579387104, -9608.682631509726, -1.7108925257214056e6, 4.332924601416521e6, -22366.683262266528, -2.5019716386377467e6, 1.0274495902259542e7, -85360.30079034246, -570025.3441737515, 4.396844346849777e6},
  {97.89747327985583, -42.659730877489224, 153.48421037904913, -1417.0620760768954, 2752.8614143665027, 138.7406469558649, -1433.6585075135881, 2857.7418952430758, 41.025109467376126, -423.680737974639, 850.3594335657173},
  {-3.282701958759534, -9.051384468245866, -12.415449742258042, 55.4716447709787, -106.05109938966335, -11.953044553690658, 76.80704618365418, -155.33172948098394, -3.4129261592393263, 25.572377569952536, -54.408036707740465},
  {-0.000025156429818799565, 0.000019750256942201327, -0.000018370671469295915, 0.000021886317041311973, 0.00008250240316860033, 7.157371250566708e-6, -0.000055780000112270685, 0.00019142082884072178, 5.447166261464217e-6, -0.00003220610095021982, 0.00007974016714984341},
  {43.31514709695348, 638.6332679188081, -32.85768747216059, 2415.8938269370315, -5766.875169379177, -61.85459307173841, 2953.967762459948, -8986.29057591497, -21.571435779762044, 981.2158224673428, -3239.5664895930286},
  {-0.07020209449091723, -0.16269798450687084, -0.1872514685185499, 1.138313650449945, -2.8334196304430046, -0.17137955686840617, 1.7197549338119527, -4.539717148261272, -0.049983437357548705, 0.6062072055948309, -1.682769616644546},
  {9.5988072383479, -397.05438595557433, 16.202126189517813, -1574.8286986717037, 3600.3410843831093, 27.092429659075467, -1786.482357315139, 5152.919378666511, 11.175710130033895, -577.7999423177481, 1808.730762932043},
  {-0.02989487384493607, 1.4022106448583738, -0.07356049468633846, 0.8337006542278661, 0.2240008282397391, -0.055202870001177226, 0.5667186343606578, 0.7186931973380503, -0.015507437354325743, 0.15750322779277187, 0.21076815715176228},
  {0.9974408278363099, -0.007884449714907203, -0.059046901195591035, 1.3958712396764088, -4.516631601676276, -0.05585343136869692, 1.7516580039343603, -5.990208965347804, -0.017945336522161195, 0.5965097794825992, -2.0608879367971804},
  {3931.8979897196614, -17395.758706812805, 3132.375545898835, 343965.86092361377, -1.2162565819981997e6, -70698.00600428853, 1.383907177859705e6, -3.9662761890979446e6, -60017.52423652596, 803515.1181825735, -2.091710365941658e6},
  {-40105.47653771657, 112253.0169706701, 23561.696065836168, -3.476180699403351e6, 1.137593670849482e7, 754313.1127166454, -1.308476044625268e7, 3.6444584853928134e7, 596226.612472288, -7.4277901143564405e6, 1.8928977514040343e7},
  {83208.35471266537, -191237.7264145924, -210916.2454782992, 8.71797508352568e6, -2.6914942420669552e7, -1.9889806527362722e6, 3.0888029960154563e7, -8.390870279256162e7, -1.4535031953446497e6, 1.7063528990822166e7, -4.2748659731120914e7},
};

// Per-sample coefficient block.  Psi is the full phase in h22 = A e^{-i Psi}
// (time and phase alignment folded in); tf = dPsi/df / (2 pi) in seconds.
template <class T>
struct PhenomDCoef {
  T Msec;               // total mass [s]
  T fRD, fDM, fpeak;    // Mf units
  T amp_scale;          // A = amp_scale * Mf^{-7/6} * Ahat(Mf)
  T ai[8];              // Ahat_ins = 1 + sum_j ai_j u^(j+2): 3PN SPA terms (j < 5), rho1..rho3 (j = 5..7)
  T dl[5];              // Ahat_int = sum dl_j Mf^j
  T g1, g2, g3fDM;      // Ahat_mrd = g1 g3fDM / ((Mf-fRD)^2 + g3fDM^2) exp(-g2 (Mf-fRD)/g3fDM)
  T pin[12];            // Psi_ins = u^-5 sum pin_j u^j + (lg0 + lg1 u) ln u
  T lg0, lg1;
  T pint[4];            // Psi_int = pint0 + pint1 Mf + pint2 Mf^-3 + pint3 ln Mf
  T pm[6];              // Psi_mrd = pm0 + pm1 Mf + pm2/Mf + pm3 Mf^{3/4} + pm4 atan((Mf - pm5)/fDM)
  T tscale;             // Msec / (2 pi)
  T pfac, cfac;         // (1 + cos^2 i)/2, cos i
  T af, erad, eta, v2;  // remnant spin, radiated energy, symmetric mass ratio, amplitude collocation value
};

template <class T>
PES_HD T phenom_fit(int w, const T& eta, const T& xi) {
  const double* c = kPhenomFits[w];
  T eta2 = eta * eta;
  return c[0] + c[1] * eta + xi * (c[2] + c[3] * eta + c[4] * eta2) +
         xi * xi * ((c[5] + c[6] * eta + c[7] * eta2) + xi * (c[8] + c[9] * eta + c[10] * eta2));
}

// Phase and its Mf-derivative from the coefficient block (region by Mf).
template <class T>
PES_HD void phenomd_phase(const PhenomDCoef<T>& c, const T& Mf, const T& u, T& psi, T& dpsi) {
  if (Mf < kPhiJoinIns) {
    T lu = dlog(u);
    // Horner for P(u) and R(u) = sum pin_j (j-5)/3 u^j
    T P = c.pin[11], R = c.pin[11] * 2.0;
#pragma unroll
    for (int j = 10; j >= 0; --j) {
      P = P * u + c.pin[j];
      R = R * u + c.pin[j] * ((j - 5) / 3.0);
    }
    T iu = 1.0 / u;
    T iu2 = iu * iu;
    T iu4 = iu2 * iu2;
    T iu5 = iu4 * iu;
    psi = P * iu5 + (c.lg0 + c.lg1 * u) * lu;
    dpsi = R * iu4 * iu4 + (c.lg1 * (lu + 1.0) * (1.0 / 3.0)) * iu2 + c.lg0 * (1.0 / 3.0) * iu2 * iu;
  } else if (Mf < 0.5 * c.fRD) {
    T iMf = 1.0 / Mf;
    T iMf3 = iMf * iMf * iMf;
    psi = c.pint[0] + c.pint[1] * Mf + c.pint[2] * iMf3 + c.pint[3] * (3.0 * dlog(u));
    dpsi = c.pint[1] - 3.0 * c.pint[2] * iMf3 * iMf + c.pint[3] * iMf;
  } else {
    T iMf = 1.0 / Mf;
    T q = dsqrt(dsqrt(Mf));  // Mf^{1/4}
    T x = Mf - c.pm[5];
    psi = c.pm[0] + c.pm[1] * Mf + c.pm[2] * iMf + c.pm[3] * (q * q * q) + c.pm[4] * datan(x / c.fDM);
    dpsi = c.pm[1] - c.pm[2] * iMf * iMf + 0.75 * c.pm[3] / q + c.pm[4] * c.fDM / (c.fDM * c.fDM + x * x);
  }
}

template <class T>
PES_HD T phenomd_amphat(const PhenomDCoef<T>& c, const T& Mf, const T& u) {
  if (Mf < kAmpJoinIns) {
    T u2 = u * u;
    return 1.0 + u2 * (c.ai[0] + u * (c.ai[1] + u * (c.ai[2] + u * (c.ai[3] + u * (c.ai[4] +
                       u * (c.ai[5] + u * (c.ai[6] + u * c.ai[7])))))));
  }
  if (Mf >= c.fpeak) {
    T x = Mf - c.fRD;
    return c.g1 * c.g3fDM / (x * x + c.g3fDM * c.g3fDM) * dexp(-c.g2 * x / c.g3fDM);
  }
  return c.dl[0] + Mf * (c.dl[1] + Mf * (c.dl[2] + Mf * (c.dl[3] + Mf * c.dl[4])));
}

// Amplitude A(f), phase Psi(f) and t(f) of h22 at Mf (caller checks the cut).
template <class T>
PES_HD void phenomd_eval(const PhenomDCoef<T>& c, const T& Mf, T& amp, T& psi, T& tf) {
  T u = dcbrt(Mf);
  T dpsi;
  phenomd_phase(c, Mf, u, psi, dpsi);
  tf = c.tscale * dpsi;
  amp = c.amp_scale / (Mf * dsqrt(u)) * phenomd_amphat(c, Mf, u);
}

// Ahat at f_peak and the jump of d^2 Ahat / dMf^2 there: the intermediate
// polynomial and the merger-ringdown Lorentzian join with C1 continuity only.
template <class T>
PES_HD void amp_peak_jump(const PhenomDCoef<T>& c, T& ahat_pk, T& jump) {
  const T fp = c.fpeak;
  const T x = fp - c.fRD, a = c.g3fDM;
  const T D = x * x + a * a;
  const T A = c.g1 * a / D * dexp(-c.g2 * x / a);
  const T L1 = -c.g2 / a - 2.0 * x / D;
  const T L2 = -2.0 * (a * a - x * x) / (D * D);
  const T d2m = A * (L1 * L1 + L2);
  const T d2i = 2.0 * c.dl[2] + fp * (6.0 * c.dl[3] + 12.0 * c.dl[4] * fp);
  ahat_pk = A;
  jump = d2m - d2i;
}

template <class T>
PES_HD void solve5(T A[5][5], T b[5], T x[5]) {
  for (int col = 0; col < 5; ++col) {
    int piv = col;
    for (int r = col + 1; r < 5; ++r)
      if (dabs(val(A[r][col])) > dabs(val(A[piv][col]))) piv = r;
    if (piv != col) {
      for (int j = 0; j < 5; ++j) { T t = A[col][j]; A[col][j] = A[piv][j]; A[piv][j] = t; }
      T t = b[col]; b[col] = b[piv]; b[piv] = t;
    }
    for (int r = col + 1; r < 5; ++r) {
      T m = A[r][col] / A[col][col];
      for (int j = col; j < 5; ++j) A[r][j] = A[r][j] - m * A[col][j];
      b[r] = b[r] - m * b[col];
    }
  }
  for (int r = 4; r >= 0; --r) {
    T s = b[r];
    for (int j = r + 1; j < 5; ++j) s = s - A[r][j] * x[j];
    x[r] = s / A[r][r];
  }
}

// Build the coefficient block from the 11-parameter vector (see the C header).
template <class T>
PES_HD void phenomd_setup(const T* th, double f_ref, PhenomDCoef<T>& c) {
  const T one = lift<T>(1.0);
  T Mc = dexp(th[0]);
  T q = th[1];
  T chi1 = th[2], chi2 = th[3];
  T opq = one + q;
  T eta = q / (opq * opq);
  T M = Mc * dpow(eta, -0.6);
  T m1 = q / opq, m2 = one / opq;
  T seta = (q - 1.0) / opq;
  T eta2 = eta * eta, eta3 = eta2 * eta;
  c.Msec = M * kMTSun;
  c.tscale = c.Msec * (1.0 / (2.0 * kPi));
  T chipn = m1 * chi1 + m2 * chi2 - (38.0 / 113.0) * eta * (chi1 + chi2);
  T xi = chipn - 1.0;
  // remnant spin and radiated energy (Husa et al. 2016)
  T s = m1 * m1 * chi1 + m2 * m2 * chi2;
  T af = eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * eta2 -
                13.180949901606242 * eta3 +
                s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) +
                     s * ((0.1014665242971878 - 2.0967746996832157 * eta) +
                          s * ((-1.3546806617824356 + 4.108962025369336 * eta) +
                               s * (-0.8676969352555539 + 2.064046835273906 * eta)))));
  T sn = s / (m1 * m1 + m2 * m2);
  T erad = ((0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2 +
             3.352411249771192 * eta3) * eta *
            (1.0 + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * sn)) /
           (1.0 + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * sn);
  // (2,2,0) quasi-normal mode of the remnant (mass 1 - E_rad, spin af)
  T wR, wI;
  qnm_interp<T>(0, af, wR, wI);
  c.fRD = wR / (2.0 * kPi) / (one - erad);
  c.fDM = wI / (2.0 * kPi) / (one - erad);
  T v2 = phenom_fit(kFV2, eta, xi);
  c.af = af;
  c.erad = erad;
  c.eta = eta;
  c.v2 = v2;
  c.g1 = phenom_fit(kFG1, eta, xi);
  c.g2 = phenom_fit(kFG2, eta, xi);
  T g3 = phenom_fit(kFG3, eta, xi);
  c.g3fDM = g3 * c.fDM;
  if (val(c.g2) <= 1.0)
    c.fpeak = dabs(c.fRD + c.fDM * g3 * (dsqrt(one - c.g2 * c.g2) - 1.0) / c.g2);
  else
    c.fpeak = dabs(c.fRD - c.fDM * g3 / c.g2);
  // 3PN SPA amplitude of the inspiral in powers of u = Mf^{1/3}
  const double pi13 = ::cbrt(kPi), pi23 = pi13 * pi13, pi43 = kPi * pi13, pi53 = kPi * pi23, pi2 = kPi * kPi;
  T c12 = chi1 * chi1, c22 = chi2 * chi2, c1c2 = chi1 * chi2;
  T sp = one + seta, sm = one - seta;
  c.ai[0] = (-969.0 + 1804.0 * eta) * (pi23 / 672.0);
  c.ai[1] = (chi1 * (81.0 * sp - 44.0 * eta) + chi2 * (81.0 * sm - 44.0 * eta)) * (kPi / 48.0);
  c.ai[2] = (-27312085.0 - 10287648.0 * (c12 * sp + c22 * sm) +
             24.0 * (-1975055.0 + 857304.0 * (c12 + c22) - 994896.0 * c1c2) * eta + 35371056.0 * eta2) *
            (pi43 / 8128512.0);
  c.ai[3] = (chi1 * (285197.0 * sp - 4.0 * (91902.0 + 1579.0 * seta) * eta - 35632.0 * eta2) +
             chi2 * (285197.0 * sm - 4.0 * (91902.0 - 1579.0 * seta) * eta - 35632.0 * eta2) +
             42840.0 * kPi * (-1.0 + 4.0 * eta)) *
            (pi53 / 32256.0);
  c.ai[4] = (336.0 * (-3248849057.0 + 2943675504.0 * (c12 + c22) - 3339284256.0 * c1c2) * eta2 +
             324322727232.0 * eta3 +
             7.0 * (-177520268561.0 + 107414046432.0 * (c12 * sp + c22 * sm) +
                    11087290368.0 * kPi * (chi1 * sp + chi2 * sm)) -
             12.0 * eta *
                 (-545384828789.0 - 176491177632.0 * c1c2 + 77616.0 * 2610335.0 * (c12 + c22) +
                  77616.0 * 995766.0 * seta * (c12 - c22) + 5841690624.0 * kPi * (chi1 + chi2) +
                  21384760320.0 * pi2)) *
            (pi2 / 60085960704.0);
  // calibrated terms rho1 Mf^{7/3} + rho2 Mf^{8/3} + rho3 Mf^3 (Khan et al. 2016 eq. 29)
  c.ai[5] = phenom_fit(kFR1, eta, xi);
  c.ai[6] = phenom_fit(kFR2, eta, xi);
  c.ai[7] = phenom_fit(kFR3, eta, xi);
  // TaylorF2 aligned-spin phasing (3.5PN, spin-orbit to 3.5PN, 2PN spin-spin,
  // no 3PN spin-spin) plus the sigma terms, as a series in u.
  T SL = m1 * m1 * chi1 + m2 * m2 * chi2;
  T dSL = seta * (m2 * chi2 - m1 * chi1);
  T pn_sigma = (474.0 / 48.0) * eta * c1c2 + (486.0 / 96.0) * (m1 * m1 * c12 + m2 * m2 * c22);
  T pn_gamma = (554345.0 / 1134.0 + (110.0 / 9.0) * eta) * SL + (13915.0 / 84.0 - (10.0 / 3.0) * eta) * dSL;
  T pfaN = 3.0 / (128.0 * eta);
  T a[8];
  a[0] = one;
  a[1] = lift<T>(0.0);
  a[2] = (5.0 / 9.0) * (743.0 / 84.0 + 11.0 * eta);
  a[3] = -16.0 * kPi + (188.0 / 3.0) * SL + 25.0 * dSL;
  a[4] = (5.0 / 72.0) * (3058.673 / 7.056 + (5429.0 / 7.0) * eta + 617.0 * eta2) - 10.0 * pn_sigma;
  T v5 = (5.0 / 9.0) * kPi * (7729.0 / 84.0 - 13.0 * eta) - pn_gamma;
  T vl5 = (5.0 / 3.0) * kPi * (7729.0 / 84.0 - 13.0 * eta) - 3.0 * pn_gamma;
  T v6 = lift<T>(11583.231236531 / 4.694215680 - 640.0 / 3.0 * pi2 - 6848.0 / 21.0 * kEulerGamma -
                 6848.0 / 21.0 * 1.3862943611198906) +
         eta * (-15737.765635 / 3.048192 + 2255.0 / 12.0 * pi2) + eta2 * (76055.0 / 1728.0) -
         eta3 * (127825.0 / 1296.0) + (kPi / 3.0) * (3760.0 * SL + 1490.0 * dSL);
  const double vl6 = -6848.0 / 21.0;
  a[7] = kPi * (77096675.0 / 254016.0 + (378515.0 / 1512.0) * eta - (74045.0 / 756.0) * eta2) +
         (-8980424995.0 / 762048.0 + (6586595.0 / 756.0) * eta - (305.0 / 36.0) * eta2) * SL -
         (170978035.0 / 48384.0 - (2876425.0 / 672.0) * eta - (4735.0 / 144.0) * eta2) * dSL;
  // v = pi^{1/3} u: pin_k = pfaN (a_k + vl_k ln pi^{1/3}) pi^{(k-5)/3}; ln v = ln pi^{1/3} + ln u
  const double lnpi13 = ::log(kPi) / 3.0;
  T pin[12];
  pin[0] = pfaN * (1.0 / pi53);
  pin[1] = lift<T>(0.0);
  pin[2] = pfaN * a[2] * (1.0 / kPi);
  pin[3] = pfaN * a[3] * (1.0 / pi23);
  pin[4] = pfaN * a[4] * (1.0 / pi13);
  pin[5] = pfaN * (v5 + vl5 * lnpi13) - 0.25 * kPi;
  pin[6] = pfaN * (v6 + vl6 * lnpi13) * pi13;
  pin[7] = pfaN * a[7] * pi23;
  T s1 = phenom_fit(kFS1, eta, xi), s2 = phenom_fit(kFS2, eta, xi), s3 = phenom_fit(kFS3, eta, xi),
    s4 = phenom_fit(kFS4, eta, xi);
  T ieta = one / eta;
  pin[8] = s1 * ieta;
  pin[9] = 0.75 * s2 * ieta;
  pin[10] = 0.6 * s3 * ieta;
  pin[11] = 0.5 * s4 * ieta;
#pragma unroll
  for (int j = 0; j < 12; ++j) c.pin[j] = pin[j];
  c.lg0 = pfaN * vl5;
  c.lg1 = pfaN * vl6 * pi13;
  T b1 = phenom_fit(kFB1, eta, xi), b2 = phenom_fit(kFB2, eta, xi), b3 = phenom_fit(kFB3, eta, xi);
  c.pint[0] = lift<T>(0.0);
  c.pint[1] = b1 * ieta;
  c.pint[2] = -b3 * ieta * (1.0 / 3.0);
  c.pint[3] = b2 * ieta;
  T a1 = phenom_fit(kFA1, eta, xi), a2 = phenom_fit(kFA2, eta, xi), a3 = phenom_fit(kFA3, eta, xi),
    a4 = phenom_fit(kFA4, eta, xi), a5 = phenom_fit(kFA5, eta, xi);
  c.pm[0] = lift<T>(0.0);
  c.pm[1] = a1 * ieta;
  c.pm[2] = -a2 * ieta;
  c.pm[3] = (4.0 / 3.0) * a3 * ieta;
  c.pm[4] = a4 * ieta;
  c.pm[5] = a5 * c.fRD;
  // C1 continuity of the phase: intermediate matched at Mf = 0.018, merger-ringdown at fRD/2
  {
    T f1 = lift<T>(kPhiJoinIns);
    T u1 = dcbrt(f1);
    T pI, dI, pN, dN;
    {  // inspiral branch at the join (Mf = 0.018 itself belongs to the intermediate region)
      T lu = dlog(u1);
      T P = c.pin[11], R = c.pin[11] * 2.0;
      for (int j = 10; j >= 0; --j) { P = P * u1 + c.pin[j]; R = R * u1 + c.pin[j] * ((j - 5) / 3.0); }
      T iu = 1.0 / u1, iu2 = iu * iu, iu4 = iu2 * iu2;
      pI = P * iu4 * iu + (c.lg0 + c.lg1 * u1) * lu;
      dI = R * iu4 * iu4 + (c.lg1 * (lu + 1.0) * (1.0 / 3.0)) * iu2 + c.lg0 * (1.0 / 3.0) * iu2 * iu;
    }
    T if1 = 1.0 / f1;
    pN = c.pint[1] * f1 + c.pint[2] * if1 * if1 * if1 + c.pint[3] * dlog(f1);
    dN = c.pint[1] - 3.0 * c.pint[2] * if1 * if1 * if1 * if1 + c.pint[3] * if1;
    T C2 = dI - dN;
    T C1 = pI - pN - C2 * f1;
    c.pint[0] = C1;
    c.pint[1] = c.pint[1] + C2;
    T f2 = 0.5 * c.fRD;
    T if2 = 1.0 / f2;
    T pI2 = c.pint[0] + c.pint[1] * f2 + c.pint[2] * if2 * if2 * if2 + c.pint[3] * dlog(f2);
    T dI2 = c.pint[1] - 3.0 * c.pint[2] * if2 * if2 * if2 * if2 + c.pint[3] * if2;
    T q2 = dsqrt(dsqrt(f2));
    T x2 = f2 - c.pm[5];
    T pM = c.pm[1] * f2 + c.pm[2] * if2 + c.pm[3] * (q2 * q2 * q2) + c.pm[4] * datan(x2 / c.fDM);
    T dM = c.pm[1] - c.pm[2] * if2 * if2 + 0.75 * c.pm[3] / q2 + c.pm[4] * c.fDM / (c.fDM * c.fDM + x2 * x2);
    T C2m = dI2 - dM;
    c.pm[0] = pI2 - pM - C2m * f2;
    c.pm[1] = c.pm[1] + C2m;
  }
  // intermediate amplitude: value/derivative at 0.014 and fpeak, value v2 midway
  {
    T f1 = lift<T>(kAmpJoinIns), f3 = c.fpeak, f2 = 0.5 * (f1 + f3);
    T u1 = dcbrt(f1);
    T u12 = u1 * u1;
    T Ains = one + u12 * (c.ai[0] + u1 * (c.ai[1] + u1 * (c.ai[2] + u1 * (c.ai[3] + u1 * (c.ai[4] +
                   u1 * (c.ai[5] + u1 * (c.ai[6] + u1 * c.ai[7])))))));
    // dAhat/dMf = (1/(3u^2)) dAhat/du
    T dAdu = u1 * (2.0 * c.ai[0] + u1 * (3.0 * c.ai[1] + u1 * (4.0 * c.ai[2] + u1 * (5.0 * c.ai[3] + u1 * (6.0 * c.ai[4] +
                   u1 * (7.0 * c.ai[5] + u1 * (8.0 * c.ai[6] + u1 * 9.0 * c.ai[7])))))));
    T dAins = dAdu / (3.0 * u12);
    T x3 = f3 - c.fRD;
    T den = x3 * x3 + c.g3fDM * c.g3fDM;
    T Amrd = c.g1 * c.g3fDM / den * dexp(-c.g2 * x3 / c.g3fDM);
    T dAmrd = Amrd * (-c.g2 / c.g3fDM - 2.0 * x3 / den);
    T A[5][5], b[5];
    T fs[3] = {f1, f2, f3};
    for (int r = 0; r < 3; ++r) {
      T pw = one;
      for (int j = 0; j < 5; ++j) { A[r][j] = pw; pw = pw * fs[r]; }
    }
    T fd[2] = {f1, f3};
    for (int r = 0; r < 2; ++r) {
      A[3 + r][0] = lift<T>(0.0);
      A[3 + r][1] = one;
      A[3 + r][2] = 2.0 * fd[r];
      A[3 + r][3] = 3.0 * fd[r] * fd[r];
      A[3 + r][4] = 4.0 * fd[r] * fd[r] * fd[r];
    }
    b[0] = Ains;
    b[1] = v2;
    b[2] = Amrd;
    b[3] = dAins;
    b[4] = dAmrd;
    solve5(A, b, c.dl);
  }
  // alignment: t(fpeak) = 0 and Psi(f_ref) = -2 phi_c
  {
    T up = dcbrt(c.fpeak);
    T pp, dp;
    phenomd_phase(c, c.fpeak, up, pp, dp);
    T t0 = dp;
    T MfRef = c.Msec * f_ref;
    T ur = dcbrt(MfRef);
    T pr, dr;
    phenomd_phase(c, MfRef, ur, pr, dr);
    T shift = t0 * MfRef - pr - 2.0 * th[9];
    // fold -t0 Mf + shift into every region
    c.pin[5] = c.pin[5] + shift;
    c.pin[8] = c.pin[8] - t0;
    c.pint[0] = c.pint[0] + shift;
    c.pint[1] = c.pint[1] - t0;
    c.pm[0] = c.pm[0] + shift;
    c.pm[1] = c.pm[1] - t0;
  }
  T DLm = dexp(th[4]) * (1.0e6 * kPc);
  // 2 sqrt(5/(64 pi)) M_m M_s / D * sqrt(2 eta / 3) pi^{-1/6}
  const double amp_norm = 2.0 * ::sqrt(5.0 / (64.0 * kPi)) / ::pow(kPi, 1.0 / 6.0);
  c.amp_scale = amp_norm * (M * kMRSun) * (M * kMTSun) / DLm * dsqrt(eta * (2.0 / 3.0));
  c.pfac = 0.5 * (one + th[5] * th[5]);
  c.cfac = th[5];
}

// ------------------------------------------------------------------ IMRPhenomHM
// The six-mode model of London et al. 2018 (arXiv:1708.00404) built on the
// (2,2) IMRPhenomD block above: modes (2,2), (2,1), (3,3), (3,2), (4,4), (4,3)
// (the quasi-normal-mode table's order).  Each mode maps onto the (2,2)
// frequency f22: 2 f / m in the inspiral, Rholm f (Rholm = fRD22 / fRD_lm)
// in the ringdown; between corners at the (2,2) joins (amplitude: Mf = 0.014
// and f_peak; phase: Mf = 0.018 and fRD22 / 2) the phase map is linear and
// the amplitude map the cubic Hermite blend of the two lines (C1).
// Amplitude: beta_lm A22(f22) with beta_lm the post-Newtonian mode ratio
// |H_lm| / |H_22| sqrt(2/m) at v = (2 pi M f_b / m)^{1/3}, f_b = f below the
// amplitude map's inspiral corner f_i and f_i (2 - exp(1 - f/f_i)) above it,
// and the (2,2) amplitude's merger-ringdown width set to the mode's (Rholm
// fDM_lm in mapped frequency; intermediate collocation re-solved).  Phase: (m/2) Psi22(2f/m) below the phase map's
// first corner, (1/a) Psi22(a f + b) + c0 + c1 f between the corners,
// (1/Rholm) Psi22_MRD(Rholm f) + c0' + c1' f above (arctangent width the
// mode's), C1 throughout; plus k_lm quarter turns (the phase of H_lm).
// Polarisations: hp = sum P_lm h_lm, hc = i sum C_lm h_lm (s = -2 spherical
// harmonics at azimuth 0; (2,2) gives (1 + cos^2 i)/2 and -cos i).
constexpr int kHMModes = 6;
__device__ __constant__ static const int kHMlm[kHMModes][3] = {  // l, m, quarter turns of H_lm
    {2, 2, 0}, {2, 1, 1}, {3, 3, 3}, {3, 2, 0}, {4, 4, 2}, {4, 3, 3}};

template <class T>
struct HMMode {
  T P, C;                       // polarisation factors
  T Rholm, fDMeff, g3fDMeff;    // ringdown map slope, the mode's damping in mapped frequency
  T fpeak, dl[5];               // mapped amplitude: peak, intermediate polynomial
  T fiA, frA;                   // amplitude map corners (Mf)
  T fiP, frP, aP, bP;           // phase map
  T cI0, cI1, cR0, cR1;         // C1 constants of the phase
  T fRD;                        // the mode's ringdown frequency (Mf)
  // the mode's constants in the evaluation's scalar type (no FP64 division or
  // conversion per node when that type is float-float): 2/m, m/2, 2 pi/m and
  // the phase's quarter turns
  T tm, hm, tpm, qt;
};

// a <= b and a >= b on the values (float-float compares without leaving the FP32 pipes)
template <class T> PES_HD bool val_le(const T& a, const T& b) { return val(a) <= val(b); }
template <class T> PES_HD bool val_ge(const T& a, const T& b) { return val(a) >= val(b); }
PES_HD bool val_le(const FF& a, const FF& b) { return a <= b; }
PES_HD bool val_ge(const FF& a, const FF& b) { return a >= b; }

template <class T>
struct PhenomHMCoef {
  T eta, dlt, chis, chia;  // for the PN amplitude ratios
  T fRDmax;                // largest ringdown frequency of the modes (Mf)
  T v2;                    // the (2,2) intermediate amplitude collocation value
  T ainsf1, dainsf1;       // the (2,2) inspiral amplitude and its Mf-derivative at Mf = 0.014
  HMMode<T> md[kHMModes];
};

PES_HD double hm_fact(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}

// s = -2 spherical harmonic at azimuth 0 from cos(iota): sqrt((2l+1)/4pi) d^l_{m,2}
template <class T>
PES_HD T hm_sylm(int l, int m, const T& cosi) {
  const T ch = dsqrt(0.5 * (1.0 + cosi)), sh = dsqrt(0.5 * (1.0 - cosi));
  T sum = lift<T>(0.0);
  for (int k = 0; k <= l + m; ++k) {
    if (l + m - k < 0 || l - 2 - k < 0 || k + 2 - m < 0) continue;
    const double c = ((k & 1) ? -1.0 : 1.0) *
                     ::sqrt(hm_fact(l + m) * hm_fact(l - m) * hm_fact(l + 2) * hm_fact(l - 2)) /
                     (hm_fact(l + m - k) * hm_fact(l - 2 - k) * hm_fact(k) * hm_fact(k + 2 - m));
    T term = lift<T>(c);
    for (int e = 0; e < 2 * l + m - 2 * k - 2; ++e) term = term * ch;
    for (int e = 0; e < 2 * k + 2 - m; ++e) term = term * sh;
    sum = sum + term;
  }
  return ::sqrt((2.0 * l + 1.0) / (4.0 * kPi)) * sum;
}

// Signed PN amplitude ratio beta_lm(v) (Blanchet 2014 eq. 327; leading spin term of (2,1))
template <class T>
PES_HD T hm_pn_ratio(int k, const T& v, const PhenomHMCoef<T>& h) {
  const T v2 = v * v;
  const T h22 = 1.0 + v2 * (-107.0 / 42.0 + (55.0 / 42.0) * h.eta) + (2.0 * kPi) * (v2 * v);
  T r;
  switch (k) {
    case 0: return lift<T>(1.0);
    case 1:
      r = (1.0 / 3.0) * (h.dlt * v * (1.0 + v2 * (-17.0 / 28.0 + (5.0 / 7.0) * h.eta)) - 1.5 * (h.chia + h.dlt * h.chis) * v2);
      return r / h22 * ::sqrt(2.0);
    case 2:
      r = (0.75 * 1.0350983390135313) * h.dlt * v * (1.0 + v2 * (-4.0 + 2.0 * h.eta));  // sqrt(15/14)
      return r / h22 * ::sqrt(2.0 / 3.0);
    case 3:
      r = (0.84515425472851657 / 3.0) * v2 * (1.0 - 3.0 * h.eta);  // sqrt(5/7)
      return r / h22 * ::sqrt(2.0 / 2.0);
    case 4:
      r = (8.0 / 9.0 * 0.84515425472851657) * v2 * (1.0 - 3.0 * h.eta);
      return r / h22 * ::sqrt(2.0 / 4.0);
    default:
      r = (9.0 / (4.0 * 8.3666002653407556)) * h.dlt * v2 * v * (1.0 - 2.0 * h.eta);  // sqrt(70)
      return r / h22 * ::sqrt(2.0 / 3.0);
  }
}

// the (2,2) merger-ringdown phase ansatz (aligned coefficients) with damping fdm
template <class T>
PES_HD void hm_psi_mrd(const PhenomDCoef<T>& c, const T& fdm, const T& Mf, T& psi, T& dpsi) {
  const T iMf = 1.0 / Mf;
  const T q = dsqrt(dsqrt(Mf));
  const T x = Mf - c.pm[5];
  psi = c.pm[0] + c.pm[1] * Mf + c.pm[2] * iMf + c.pm[3] * (q * q * q) + c.pm[4] * datan(x / fdm);
  dpsi = c.pm[1] - c.pm[2] * iMf * iMf + 0.75 * c.pm[3] / q + c.pm[4] * fdm / (fdm * fdm + x * x);
}

// mode k's phase (without the quarter turns) and dPsi/dMf
template <class T>
PES_HD void hm_phase(const PhenomDCoef<T>& c, const HMMode<T>& md, int m, const T& Mf, T& psi, T& dpsi) {
  if (Mf < md.fiP) {
    const T f22 = md.tm * Mf;
    phenomd_phase<T>(c, f22, dcbrt(f22), psi, dpsi);
    psi = md.hm * psi;
  } else if (Mf < md.frP) {
    const T f22 = md.aP * Mf + md.bP;
    phenomd_phase<T>(c, f22, dcbrt(f22), psi, dpsi);
    psi = psi / md.aP + md.cI0 + md.cI1 * Mf;
    dpsi = dpsi + md.cI1;
  } else {
    hm_psi_mrd<T>(c, md.fDMeff, md.Rholm * Mf, psi, dpsi);
    psi = psi / md.Rholm + md.cR0 + md.cR1 * Mf;
    dpsi = dpsi + md.cR1;
  }
}

// mapped (2,2) amplitude hat with the mode's merger-ringdown width
template <class T>
PES_HD T hm_amphat(const PhenomDCoef<T>& c, const HMMode<T>& md, const T& Mf22, const T& u) {
  if (Mf22 < kAmpJoinIns) return phenomd_amphat<T>(c, Mf22, u);
  if (Mf22 >= md.fpeak) {
    const T x = Mf22 - c.fRD;
    return c.g1 * md.g3fDMeff / (x * x + md.g3fDMeff * md.g3fDMeff) * dexp(-c.g2 * x / md.g3fDMeff);
  }
  return md.dl[0] + Mf22 * (md.dl[1] + Mf22 * (md.dl[2] + Mf22 * (md.dl[3] + Mf22 * md.dl[4])));
}

// the amplitude's frequency map: 2 f / m below fiA, Rholm f above frA, the
// cubic Hermite blend of the two (values and slopes) between
template <class T>
PES_HD T hm_amp_map(const HMMode<T>& md, int m, const T& Mf) {
  (void)m;
  if (val_le(Mf, md.fiA)) return md.tm * Mf;
  if (val_ge(Mf, md.frA)) return md.Rholm * Mf;
  const T h = md.frA - md.fiA, s = (Mf - md.fiA) / h;
  const T s2 = s * s, s3 = s2 * s;
  return (2.0 * s3 - 3.0 * s2 + 1.0) * (md.tm * md.fiA) + (s3 - 2.0 * s2 + s) * (h * md.tm) +
         (3.0 * s2 - 2.0 * s3) * (md.Rholm * md.frA) + (s3 - s2) * (h * md.Rholm);
}

// Mode k at Mf: amplitude, phase (with the quarter turns) and t(f) [s]; the
// mapped (amplitude) frequency in *f22 for the caller's Mf = 0.2 cut.
template <class T>
PES_HD void phenomhm_eval(const PhenomDCoef<T>& c, const PhenomHMCoef<T>& h, int k, const T& Mf, T& amp, T& psi,
                          T& tf, T* f22_out) {
  const HMMode<T>& md = h.md[k];
  const int m = kHMlm[k][1];
  const T f22 = k == 0 ? Mf : hm_amp_map<T>(md, m, Mf);
  if (f22_out) *f22_out = f22;
  const T u = dcbrt(f22);
  T beta = lift<T>(1.0);
  if (k != 0) {
    const T fb = val_le(Mf, md.fiA) ? Mf : md.fiA * (2.0 - dexp(1.0 - Mf / md.fiA));
    beta = hm_pn_ratio<T>(k, dcbrt(md.tpm * fb), h);
  }
  amp = beta * (c.amp_scale / (f22 * dsqrt(u)) * hm_amphat<T>(c, md, f22, u));
  T dpsi;
  hm_phase<T>(c, md, m, Mf, psi, dpsi);
  psi = psi + md.qt;
  tf = c.tscale * dpsi;
}

// Mode k's amplitude kink: where its amplitude stops being C2 with the
// largest jump of the second derivative.  (2,2): PhenomD's f_peak
// (amp_peak_jump).  k > 0: Mf = frA, where the mapped frequency reaches the
// mode's f_peak and the amplitude map turns linear; with A = beta A0 F(f22),
// F(y) = y^(-7/6) Ahat(y), the jump of d^2 A / dMf^2 divided by
// beta A0 y^(-7/6) is Rholm^2 [Ahat''] - y''_left (Ahat' - 7/6 Ahat / y) (the
// map is C1 there, its second derivative y''_left on the Hermite side, 0
// on the linear one).  Out: the kink's Mf, Ahat there and that jump.
template <class T>
PES_HD void hm_kink(const PhenomDCoef<T>& c, const PhenomHMCoef<T>& h, int k, T& mf_pk, T& ahat_pk, T& jump) {
  if (k == 0) {
    mf_pk = c.fpeak;
    amp_peak_jump<T>(c, ahat_pk, jump);
    return;
  }
  const HMMode<T>& md = h.md[k];
  const double m = kHMlm[k][1];
  const T fp = md.fpeak, x = fp - c.fRD, a = md.g3fDMeff;
  const T D = x * x + a * a;
  const T A = c.g1 * a / D * dexp(-c.g2 * x / a);
  const T L1 = -c.g2 / a - 2.0 * x / D;
  const T L2 = -2.0 * (a * a - x * x) / (D * D);
  const T d2m = A * (L1 * L1 + L2);
  const T d2i = 2.0 * md.dl[2] + fp * (6.0 * md.dl[3] + 12.0 * md.dl[4] * fp);
  const T hh = md.frA - md.fiA;
  T ypp = lift<T>(0.0);
  if (val(hh) > 0.0)  // the Hermite blend's second derivative at its right end
    ypp = (6.0 * (2.0 / m) * md.fiA + 2.0 * (2.0 / m) * hh - 6.0 * md.Rholm * md.frA + 4.0 * md.Rholm * hh) / (hh * hh);
  mf_pk = md.frA;
  ahat_pk = A;
  jump = md.Rholm * md.Rholm * (d2m - d2i) - ypp * (A * L1 - (7.0 / 6.0) * A / fp);
}

// The modes' coefficients from the (2,2) block c (already set up from th)
// and the remnant spin af and radiated energy erad of that set-up.
template <class T>
PES_HD void phenomhm_setup(const T* th, const PhenomDCoef<T>& c, PhenomHMCoef<T>& h) {
  const T one = lift<T>(1.0);
  const T af = c.af, erad = c.erad, eta = c.eta, v2 = c.v2;
  const T q = th[1];
  h.eta = eta;
  h.dlt = (q - 1.0) / (q + 1.0);
  h.chis = 0.5 * (th[2] + th[3]);
  h.chia = 0.5 * (th[2] - th[3]);
  h.v2 = v2;
  h.fRDmax = c.fRD;
  const double nrm = 2.0 * ::sqrt(5.0 / (64.0 * kPi));
  const T f1 = lift<T>(kAmpJoinIns);
  const T u1 = dcbrt(f1);
  for (int k = 0; k < kHMModes; ++k) {
    HMMode<T>& md = h.md[k];
    const int l = kHMlm[k][0], m = kHMlm[k][1];
    md.tm = lift<T>(2.0 / m);
    md.hm = lift<T>(0.5 * m);
    md.tpm = lift<T>(2.0 * kPi / m);
    md.qt = lift<T>(kHMlm[k][2] * (0.5 * kPi));
    const T Yp = hm_sylm<T>(l, m, th[5]), Ym = hm_sylm<T>(l, -m, th[5]);
    const double sg = (l & 1) ? -1.0 : 1.0;
    md.P = (sg * Ym + Yp) * (1.0 / (2.0 * nrm));
    md.C = (sg * Ym - Yp) * (1.0 / (2.0 * nrm));
    T wR, wI;
    qnm_interp<T>(k, af, wR, wI);
    md.fRD = wR / (2.0 * kPi) / (one - erad);
    const T fDMlm = wI / (2.0 * kPi) / (one - erad);
    if (val(md.fRD) > val(h.fRDmax)) h.fRDmax = md.fRD;
    if (k == 0) {  // the (2,2) mode is PhenomD's, bit for bit
      md.fRD = c.fRD;
      md.Rholm = one;
      md.fDMeff = c.fDM;
      md.g3fDMeff = c.g3fDM;
      md.fpeak = c.fpeak;
      for (int j = 0; j < 5; ++j) md.dl[j] = c.dl[j];
      md.fiA = f1;
      md.frA = c.fpeak;
      md.fiP = lift<T>(kPhiJoinIns);
      md.frP = 0.5 * c.fRD;
      md.aP = one;
      md.bP = lift<T>(0.0);
      md.cI0 = md.cI1 = md.cR0 = md.cR1 = lift<T>(0.0);
      continue;
    }
    md.Rholm = c.fRD / md.fRD;
    md.fDMeff = md.Rholm * fDMlm;
    const T g3 = c.g3fDM / c.fDM;
    md.g3fDMeff = g3 * md.fDMeff;
    if (val(c.g2) <= 1.0)
      md.fpeak = dabs(c.fRD + md.fDMeff * g3 * (dsqrt(one - c.g2 * c.g2) - 1.0) / c.g2);
    else
      md.fpeak = dabs(c.fRD - md.fDMeff * g3 / c.g2);
    // intermediate amplitude with the mode's merger-ringdown
    {
      const T f3 = md.fpeak, f2 = 0.5 * (f1 + f3);
      const T u12 = u1 * u1;
      const T Ains = one + u12 * (c.ai[0] + u1 * (c.ai[1] + u1 * (c.ai[2] + u1 * (c.ai[3] + u1 * (c.ai[4] +
                     u1 * (c.ai[5] + u1 * (c.ai[6] + u1 * c.ai[7])))))));
      const T dAdu = u1 * (2.0 * c.ai[0] + u1 * (3.0 * c.ai[1] + u1 * (4.0 * c.ai[2] + u1 * (5.0 * c.ai[3] + u1 * (6.0 * c.ai[4] +
                     u1 * (7.0 * c.ai[5] + u1 * (8.0 * c.ai[6] + u1 * 9.0 * c.ai[7])))))));
      const T dAins = dAdu / (3.0 * u12);
      const T x3 = f3 - c.fRD;
      const T den = x3 * x3 + md.g3fDMeff * md.g3fDMeff;
      const T Amrd = c.g1 * md.g3fDMeff / den * dexp(-c.g2 * x3 / md.g3fDMeff);
      const T dAmrd = Amrd * (-c.g2 / md.g3fDMeff - 2.0 * x3 / den);
      T A[5][5], b[5];
      const T fs[3] = {f1, f2, f3};
      for (int r = 0; r < 3; ++r) {
        T pw = one;
        for (int j = 0; j < 5; ++j) { A[r][j] = pw; pw = pw * fs[r]; }
      }
      const T fd[2] = {f1, f3};
      for (int r = 0; r < 2; ++r) {
        A[3 + r][0] = lift<T>(0.0);
        A[3 + r][1] = one;
        A[3 + r][2] = 2.0 * fd[r];
        A[3 + r][3] = 3.0 * fd[r] * fd[r];
        A[3 + r][4] = 4.0 * fd[r] * fd[r] * fd[r];
      }
      b[0] = Ains;
      b[1] = v2;
      b[2] = Amrd;
      b[3] = dAins;
      b[4] = dAmrd;
      solve5(A, b, md.dl);
    }
    // maps
    md.fiA = (0.5 * m) * f1;
    md.frA = md.fpeak / md.Rholm;
    md.fiP = lift<T>((0.5 * m) * kPhiJoinIns);
    md.frP = (0.5 * c.fRD) / md.Rholm;
    md.aP = (0.5 * c.fRD - kPhiJoinIns) / (md.frP - md.fiP);
    md.bP = kPhiJoinIns - md.aP * md.fiP;
    // C1 matching of the phase at fiP and frP
    md.cI0 = md.cI1 = md.cR0 = md.cR1 = lift<T>(0.0);
    T v1, d1, va, da;
    {
      const T f22 = (2.0 / m) * md.fiP;
      phenomd_phase<T>(c, f22, dcbrt(f22), v1, d1);
      v1 = (0.5 * m) * v1;
    }
    {
      const T f22 = md.aP * md.fiP + md.bP;
      phenomd_phase<T>(c, f22, dcbrt(f22), va, da);
      va = va / md.aP;
    }
    md.cI1 = d1 - da;
    md.cI0 = v1 - va - md.cI1 * md.fiP;
    T vb, db, vr, dr;
    {
      const T f22 = md.aP * md.frP + md.bP;
      phenomd_phase<T>(c, f22, dcbrt(f22), vb, db);
      vb = vb / md.aP + md.cI0 + md.cI1 * md.frP;
      db = db + md.cI1;
    }
    hm_psi_mrd<T>(c, md.fDMeff, md.Rholm * md.frP, vr, dr);
    vr = vr / md.Rholm;
    md.cR1 = db - dr;
    md.cR0 = vb - vr - md.cR1 * md.frP;
  }
}

}  // namespace pes
