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

// ------------------------------------------------------------------ IMRPhenomD
constexpr double kAmpJoinIns = 0.014;  // Mf of the inspiral/intermediate amplitude join
constexpr double kPhiJoinIns = 0.018;  // Mf of the inspiral/intermediate phase join
constexpr double kMfCut = 0.2;         // PhenomD is zero above Mf = 0.2

// Coefficient fits (Khan et al. 2016 Table V): v2, gamma1..3, sigma1..4, beta1..3, alpha1..5;
// value = c0 + c1 eta + xi (c2 + c3 eta + c4 eta^2) + xi^2 (c5 + ...) + xi^3 (c8 + ...), xi = chi_PN - 1.
enum { kFV2, kFG1, kFG2, kFG3, kFS1, kFS2, kFS3, kFS4, kFB1, kFB2, kFB3, kFA1, kFA2, kFA3, kFA4, kFA5, kFCount };
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
};

// Per-sample coefficient block.  Psi is the full phase in h22 = A e^{-i Psi}
// (time and phase alignment folded in); tf = dPsi/df / (2 pi) in seconds.
template <class T>
struct PhenomDCoef {
  T Msec;               // total mass [s]
  T fRD, fDM, fpeak;    // Mf units
  T amp_scale;          // A = amp_scale * Mf^{-7/6} * Ahat(Mf)
  T ai[5];              // Ahat_ins = 1 + ai0 u^2 + ai1 u^3 + ai2 u^4 + ai3 u^5 + ai4 u^6
  T dl[5];              // Ahat_int = sum dl_j Mf^j
  T g1, g2, g3fDM;      // Ahat_mrd = g1 g3fDM / ((Mf-fRD)^2 + g3fDM^2) exp(-g2 (Mf-fRD)/g3fDM)
  T pin[12];            // Psi_ins = u^-5 sum pin_j u^j + (lg0 + lg1 u) ln u
  T lg0, lg1;
  T pint[4];            // Psi_int = pint0 + pint1 Mf + pint2 Mf^-3 + pint3 ln Mf
  T pm[6];              // Psi_mrd = pm0 + pm1 Mf + pm2/Mf + pm3 Mf^{3/4} + pm4 atan((Mf - pm5)/fDM)
  T tscale;             // Msec / (2 pi)
  T pfac, cfac;         // (1 + cos^2 i)/2, cos i
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
    return 1.0 + u2 * (c.ai[0] + u * (c.ai[1] + u * (c.ai[2] + u * (c.ai[3] + u * c.ai[4]))));
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
  // (2,2,0) quasi-normal mode: Berti, Cardoso & Will (2006) fits
  T om = one - af;
  T wR = 1.5251 - 1.1568 * dpow(om, 0.1292);
  T Qf = 0.7 + 1.4187 * dpow(om, -0.4990);
  T mscale = 1.0 / ((2.0 * kPi) * (one - erad));
  c.fRD = wR * mscale;
  c.fDM = wR / (2.0 * Qf) * mscale;
  T v2 = phenom_fit(kFV2, eta, xi);
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
    T Ains = one + u12 * (c.ai[0] + u1 * (c.ai[1] + u1 * (c.ai[2] + u1 * (c.ai[3] + u1 * c.ai[4]))));
    // dAhat/dMf = (1/(3u^2)) dAhat/du
    T dAdu = u1 * (2.0 * c.ai[0] + u1 * (3.0 * c.ai[1] + u1 * (4.0 * c.ai[2] + u1 * (5.0 * c.ai[3] + u1 * 6.0 * c.ai[4]))));
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

}  // namespace pes
