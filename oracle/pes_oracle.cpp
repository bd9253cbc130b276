// CPU FP64 oracle of the pespace frequency-domain response / TDI / Whittle path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product in
// pespace_gb300/; the product never links, loads or calls it.  It is a plain,
// sequential restatement of the reference algorithm (citations are paths inside
// the nnrui/pespace project) plus IMRPhenomD restated from the published papers
// (Husa et al. 2016, arXiv:1508.07250; Khan et al. 2016, arXiv:1508.07253),
// which the reference does not contain.  Everything is templated on the scalar
// type so that a forward-mode dual number gives exact parameter gradients.
//
// Compiled with -ffp-contract=off so that x86 and Arm hosts give the same bits.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>

// Kerr quasi-normal-mode table (model data shared with the CUDA kernels)
#define PES_QNM_STORAGE static const
#include "../pespace_gb300/csrc/pes_qnm_table.h"
#endif

namespace orc {

// pespace/utils/constants.py:28-57
constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double C_SI = 299792458.0;
constexpr double MRSUN_SI = 1.476625038050124729627979840144936351e3;
constexpr double MTSUN_SI = 4.925490947641266978197229498498379006e-6;
constexpr double YEAR_SI = 31557600.0;
constexpr double AU_SI = 149597870700.0;
constexpr double PC_SI = 3.085677581491367e16;
constexpr double EULER_GAMMA = 0.5772156649015329;
constexpr double AU_SEC = AU_SI / C_SI;  // orbit.py:12

// ----------------------------------------------------------------- dual numbers
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
  Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0.0; }  // NOLINT
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v / b.v; double ib = 1.0 / b.v; for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib; return r; }
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v += a; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { Dual<N> r = -b; r.v += a; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N> inline Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { a = a * b; return a; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
template <int N> inline bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> inline bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> inline bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> inline bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> inline bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> inline bool operator==(const Dual<N>& a, double b) { return a.v == b; }
template <int N> inline Dual<N> chain(const Dual<N>& a, double fv, double dfv) { Dual<N> r; r.v = fv; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * dfv; return r; }
template <int N> inline Dual<N> sin(const Dual<N>& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
template <int N> inline Dual<N> cos(const Dual<N>& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
template <int N> inline Dual<N> exp(const Dual<N>& a) { double e = std::exp(a.v); return chain(a, e, e); }
template <int N> inline Dual<N> log(const Dual<N>& a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) { double s = std::sqrt(a.v); return chain(a, s, 0.5 / s); }
template <int N> inline Dual<N> cbrt(const Dual<N>& a) { double c = std::cbrt(a.v); return chain(a, c, 1.0 / (3.0 * c * c)); }
template <int N> inline Dual<N> atan(const Dual<N>& a) { return chain(a, std::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
template <int N> inline Dual<N> asin(const Dual<N>& a) { return chain(a, std::asin(a.v), 1.0 / std::sqrt(1.0 - a.v * a.v)); }
template <int N> inline Dual<N> pow(const Dual<N>& a, double p) { double q = std::pow(a.v, p); return chain(a, q, p * std::pow(a.v, p - 1.0)); }
template <int N> inline Dual<N> fabs(const Dual<N>& a) { return a.v < 0 ? -a : a; }

using std::sin; using std::cos; using std::exp; using std::log; using std::sqrt;
using std::cbrt; using std::atan; using std::asin; using std::pow; using std::fabs;

inline double val(double x) { return x; }
template <int N> inline double val(const Dual<N>& x) { return x.v; }

template <class T>
struct Cx {
  T re, im;
};
template <class T> inline Cx<T> cadd(const Cx<T>& a, const Cx<T>& b) { return {a.re + b.re, a.im + b.im}; }
template <class T> inline Cx<T> csub(const Cx<T>& a, const Cx<T>& b) { return {a.re - b.re, a.im - b.im}; }
// taichi.math.cmul order: (x0*y0 - x1*y1, x0*y1 + x1*y0)
template <class T> inline Cx<T> cmul(const Cx<T>& a, const Cx<T>& b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <class T, class S> inline Cx<T> cscale(const S& s, const Cx<T>& a) { return {s * a.re, s * a.im}; }

// ----------------------------------------------------------------- orbits
// POD orbit description; filled from Python (oracle/fdpath.py).
struct OrbitDesc {
  int32_t kind;  // 0 heliocentric (orbit.py:155-241), 1 geocentric (orbit.py:67-152)
  int32_t pad;
  double arm_sec;
  double rotation_initial, revolution_initial;
  double omega_revolution;
  double r_sec;  // heliocentric r' = L/(2 sqrt3) (orbit.py:192); geocentric L/sqrt3 (orbit.py:130)
  double omega_rotation;
  double slam_ref, clam_ref, sbeta_ref, cbeta_ref;
  double ck[3], sk[3];
};

// n[i] = n_{i+1}, x[i] = x_{i+1}; orbit.py:362-419 (heliocentric), 260-322 (geocentric)
template <class T>
void constellation(const OrbitDesc& o, const T& t, T n[3][3], T x[3][3]) {
  T xd[3][3];
  T x0[3];
  if (o.kind == 0) {
    T alpha = o.omega_revolution * t + o.revolution_initial;
    T ca = cos(alpha), sa = sin(alpha);
    T ca2 = ca * ca, sa2 = sa * sa;
    const double sqrt3 = std::sqrt(3.0);
    for (int k = 0; k < 3; ++k) {
      xd[k][0] = o.r_sec * (sa * ca * o.sk[k] - (1.0 + sa2) * o.ck[k]);
      xd[k][1] = o.r_sec * (sa * ca * o.ck[k] - (1.0 + ca2) * o.sk[k]);
      xd[k][2] = o.r_sec * (-sqrt3 * (ca * o.ck[k] + sa * o.sk[k]));
    }
    x0[0] = ca * AU_SEC;
    x0[1] = sa * AU_SEC;
    x0[2] = T(0.0);
  } else {
    T alpha = o.omega_revolution * t + o.revolution_initial;
    T kap[3];
    kap[0] = o.omega_rotation * t + o.rotation_initial;
    kap[1] = kap[0] + 2 * PI / 3;
    kap[2] = kap[1] + 2 * PI / 3;
    for (int k = 0; k < 3; ++k) {
      T ck = cos(kap[k]), sk = sin(kap[k]);
      xd[k][0] = o.r_sec * (o.sbeta_ref * o.clam_ref * sk + o.slam_ref * ck);
      xd[k][1] = o.r_sec * (o.sbeta_ref * o.slam_ref * sk - o.clam_ref * ck);
      xd[k][2] = o.r_sec * (-o.cbeta_ref * sk);
    }
    x0[0] = cos(alpha) * AU_SEC;
    x0[1] = sin(alpha) * AU_SEC;
    x0[2] = T(0.0);
  }
  for (int j = 0; j < 3; ++j) {
    n[0][j] = (xd[2][j] - xd[1][j]) / o.arm_sec;  // n1: 2 -> 3
    n[1][j] = (xd[0][j] - xd[2][j]) / o.arm_sec;  // n2: 3 -> 1
    n[2][j] = (xd[1][j] - xd[0][j]) / o.arm_sec;  // n3: 1 -> 2
    for (int k = 0; k < 3; ++k) x[k][j] = xd[k][j] + x0[j];
  }
}

// antenna.py:42-87 (polarisation tensors) and 90-114 (propagation vector);
// latitude given by its sine and cosine.
template <class T>
void polarization(const T& lam, const T& sb, const T& cb, const T& psi, T P[3][3], T X[3][3], T k[3]) {
  T sl = sin(lam), cl = cos(lam), sp = sin(psi), cp = cos(psi);
  T p[3] = {sl * cp - cl * sb * sp, -cl * cp - sl * sb * sp, cb * sp};
  T q[3] = {-sl * sp - cl * sb * cp, cl * sp - sl * sb * cp, cb * cp};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      P[i][j] = p[i] * p[j] - q[i] * q[j];
      X[i][j] = p[i] * q[j] + q[i] * p[j];
    }
  k[0] = -cb * cl;
  k[1] = -cb * sl;
  k[2] = -sb;
}

template <class T>
inline T nMn(const T n[3], const T M[3][3]) {
  T r = T(0.0);
  for (int j = 0; j < 3; ++j) {
    T nm = n[0] * M[0][j] + n[1] * M[1][j] + n[2] * M[2][j];
    r = r + nm * n[j];
  }
  return r;
}
template <class T>
inline T dot3(const T a[3], const T b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// utils.py:60-79
template <class T>
inline T sinc(const T& x) { return (val(x) == 0.0) ? T(1.0) : sin(x) / x; }

// antenna.py:462-543: six single-link responses at one frequency for one
// (already time-shifted) mode.  Order: 12, 21, 23, 32, 31, 13.
template <class T>
void links_at_f(const OrbitDesc& o, double f, const Cx<T>& hp, const Cx<T>& hc, const T& tf,
                const T P[3][3], const T X[3][3], const T k[3], Cx<T> out[6]) {
  T n[3][3], x[3][3];
  constellation(o, tf, n, x);
  const double arm = o.arm_sec;
  Cx<T> nh[3];
  for (int i = 0; i < 3; ++i) {
    T fp = nMn(n[i], P), fc = nMn(n[i], X);
    nh[i] = cadd(cscale(fp, hp), cscale(fc, hc));
  }
  T kn[3] = {dot3(k, n[0]), dot3(k, n[1]), dot3(k, n[2])};
  T s12[3], s23[3], s31[3];
  for (int j = 0; j < 3; ++j) {
    s12[j] = x[0][j] + x[1][j];
    s23[j] = x[1][j] + x[2][j];
    s31[j] = x[2][j] + x[0][j];
  }
  T kx12 = dot3(k, s12), kx23 = dot3(k, s23), kx31 = dot3(k, s31);
  const double pifL = PI * f * arm;
  T sinc32 = sinc(pifL * (1.0 - kn[0]));
  T sinc23 = sinc(pifL * (1.0 + kn[0]));
  T sinc13 = sinc(pifL * (1.0 - kn[1]));
  T sinc31 = sinc(pifL * (1.0 + kn[1]));
  T sinc21 = sinc(pifL * (1.0 - kn[2]));
  T sinc12 = sinc(pifL * (1.0 + kn[2]));
  const double ce = -PI * f;
  T a12 = ce * (arm + kx12), a23 = ce * (arm + kx23), a31 = ce * (arm + kx31);
  Cx<T> e12{cos(a12), sin(a12)}, e23{cos(a23), sin(a23)}, e31{cos(a31), sin(a31)};
  Cx<T> pre{T(-0.0), T(-pifL)};
  Cx<T> b3 = cmul(cmul(pre, nh[2]), e12);
  Cx<T> b1 = cmul(cmul(pre, nh[0]), e23);
  Cx<T> b2 = cmul(cmul(pre, nh[1]), e31);
  out[0] = cscale(sinc12, b3);
  out[1] = cscale(sinc21, b3);
  out[2] = cscale(sinc23, b1);
  out[3] = cscale(sinc32, b1);
  out[4] = cscale(sinc31, b2);
  out[5] = cscale(sinc13, b2);
}

// antenna.py:429-458: time shift by tc, then sum the modes' links.
template <class T>
void response_at_f(const OrbitDesc& o, double f, int nmodes, const Cx<T>* hp, const Cx<T>* hc, const T* tf,
                   const T& tc, const T P[3][3], const T X[3][3], const T k[3], Cx<T> out[6]) {
  T arg = -2.0 * PI * f * tc;
  Cx<T> ts{cos(arg), sin(arg)};
  for (int l = 0; l < 6; ++l) out[l] = Cx<T>{T(0.0), T(0.0)};
  for (int m = 0; m < nmodes; ++m) {
    Cx<T> lk[6];
    links_at_f(o, f, cmul(hp[m], ts), cmul(hc[m], ts), tf[m] + tc, P, X, k, lk);
    if (nmodes == 1) {
      for (int l = 0; l < 6; ++l) out[l] = lk[l];
    } else {
      for (int l = 0; l < 6; ++l) out[l] = cadd(out[l], lk[l]);
    }
  }
}

// tdi.py:1683-1703 (delay factor, generation prefactor) and 1705-1793 (X/Y/Z, A/E/T)
template <class T>
void tdi_at_f(double f, double arm, int gen20, int orth, const Cx<T> L[6], Cx<T> out[3]) {
  const double s = -2.0 * PI * f * arm;
  Cx<double> D{std::cos(s), std::sin(s)};
  Cx<double> D2 = cmul(D, D);
  Cx<double> Pf;
  if (!gen20) {
    Pf = Cx<double>{1.0 - D2.re, 0.0 - D2.im};
  } else {
    Cx<double> D4 = cmul(D2, D2);
    Cx<double> D6 = cmul(D2, D4);
    Pf = Cx<double>{1.0 - D2.re - D4.re + D6.re, 0.0 - D2.im - D4.im + D6.im};
  }
  Cx<T> Dt{T(D.re), T(D.im)}, Pt{T(Pf.re), T(Pf.im)};
  // L: 0=12 1=21 2=23 3=32 4=31 5=13
  Cx<T> Xc = cmul(Pt, cadd(csub(L[5], L[0]), cmul(Dt, csub(L[4], L[1]))));
  Cx<T> Yc = cmul(Pt, cadd(csub(L[1], L[2]), cmul(Dt, csub(L[0], L[3]))));
  Cx<T> Zc = cmul(Pt, cadd(csub(L[3], L[4]), cmul(Dt, csub(L[2], L[5]))));
  if (orth) {
    const double r2 = std::sqrt(2.0), r6 = std::sqrt(6.0), r3 = std::sqrt(3.0);
    out[0] = Cx<T>{(Zc.re - Xc.re) / r2, (Zc.im - Xc.im) / r2};
    out[1] = Cx<T>{(Xc.re - 2.0 * Yc.re + Zc.re) / r6, (Xc.im - 2.0 * Yc.im + Zc.im) / r6};
    out[2] = Cx<T>{(Xc.re + Yc.re + Zc.re) / r3, (Xc.im + Yc.im + Zc.im) / r3};
  } else {
    out[0] = Xc;
    out[1] = Yc;
    out[2] = Zc;
  }
}

// ----------------------------------------------------------------- IMRPhenomD
// Phenomenological coefficient fits, Khan et al. 2016 (arXiv:1508.07253) Table V
// (the amplitude collocation value v2, gamma1..3, sigma1..4, beta1..3, alpha1..5):
// value = l00 + l10 eta + xi (l01 + l11 eta + l21 eta^2) + xi^2 (l02 + l12 eta + l22 eta^2)
//       + xi^3 (l03 + l13 eta + l23 eta^2), with xi = chi_PN - 1.
enum { F_V2, F_G1, F_G2, F_G3, F_S1, F_S2, F_S3, F_S4,
       F_B1, F_B2, F_B3, F_A1, F_A2, F_A3, F_A4, F_A5, F_R1, F_R2, F_R3, F_COUNT };
static const double kFit[F_COUNT][11] = {
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
  // rho1..rho3: the calibrated inspiral amplitude terms (coefficients of Mf^{7/3}, Mf^{8/3}, Mf^3)
  {3931.8979897196614, -17395.758706812805, 3132.375545898835, 343965.86092361377, -1.2162565819981997e6, -70698.00600428853, 1.383907177859705e6, -3.9662761890979446e6, -60017.52423652596, 803515.1181825735, -2.091710365941658e6},
  {-40105.47653771657, 112253.0169706701, 23561.696065836168, -3.476180699403351e6, 1.137593670849482e7, 754313.1127166454, -1.308476044625268e7, 3.6444584853928134e7, 596226.612472288, -7.4277901143564405e6, 1.8928977514040343e7},
  {83208.35471266537, -191237.7264145924, -210916.2454782992, 8.71797508352568e6, -2.6914942420669552e7, -1.9889806527362722e6, 3.0888029960154563e7, -8.390870279256162e7, -1.4535031953446497e6, 1.7063528990822166e7, -4.2748659731120914e7},
};

template <class T>
T fit_eval(int which, const T& eta, const T& xi) {
  const double* c = kFit[which];
  T eta2 = eta * eta;
  T xi2 = xi * xi;
  T xi3 = xi2 * xi;
  return c[0] + c[1] * eta + xi * (c[2] + c[3] * eta + c[4] * eta2) + xi2 * (c[5] + c[6] * eta + c[7] * eta2) +
         xi3 * (c[8] + c[9] * eta + c[10] * eta2);
}

// Kerr quasi-normal modes: M omega = wR - i wI of mode `mode` (table order
// (2,2), (2,1), (3,3), (3,2), (4,4), (4,3)) at dimensionless spin a, from the
// natural cubic spline in u = sqrt(1 - a) through the tabulated frequencies
// (computed by Leaver's continued fractions, pespace_gb300/csrc/gen_qnm_table.py);
// a is clamped to +-PES_QNM_A_MAX.
template <class T>
void qnm_interp(int mode, const T& a, T& wR, T& wI) {
  T ac = a;
  if (val(ac) > PES_QNM_A_MAX) ac = T(PES_QNM_A_MAX);
  if (val(ac) < -PES_QNM_A_MAX) ac = T(-PES_QNM_A_MAX);
  T u = sqrt(1.0 - ac);
  int i = (int)std::floor((val(u) - PES_QNM_U0) / PES_QNM_DU);
  if (i < 0) i = 0;
  if (i > PES_QNM_NODES - 2) i = PES_QNM_NODES - 2;
  const double h = PES_QNM_DU;
  T t = (u - (PES_QNM_U0 + i * h)) / h;
  T s = 1.0 - t;
  T cA = (s * s * s - s) * (h * h / 6.0), cB = (t * t * t - t) * (h * h / 6.0);
  const double* re = kQnmTable[mode][0];
  const double* re2 = kQnmTable[mode][1];
  const double* im = kQnmTable[mode][2];
  const double* im2 = kQnmTable[mode][3];
  wR = s * re[i] + t * re[i + 1] + cA * re2[i] + cB * re2[i + 1];
  wI = s * im[i] + t * im[i + 1] + cA * im2[i] + cB * im2[i + 1];
}

// Phenomenological constants of IMRPhenomD.
constexpr double AMP_F_JOIN_INS = 0.014;
constexpr double PHI_F_JOIN_INS = 0.018;
constexpr double MF_CUT = 0.2;

template <class T>
struct PhenomD {
  T M_sec, eta, chi1, chi2, seta;
  T fRD, fDM, fpeak;
  T ampc[8];    // Mf^{2/3}, Mf, Mf^{4/3}, Mf^{5/3}, Mf^2, Mf^{7/3}, Mf^{8/3}, Mf^3
  T g1, g2, g3;
  T dl[5];      // intermediate amplitude polynomial
  T pv[8], pvl[8];  // TaylorF2 phasing coefficients (incl. 3/(128 eta))
  T s1, s2, s3, s4, b1, b2, b3, a1, a2, a3, a4, a5;
  T C1Int, C2Int, C1MRD, C2MRD;
  T t0, MfRef, phi_shift;  // Psi = Phi(Mf) - t0 (Mf - MfRef) - phi_shift
  T amp_scale;              // h22 = amp_scale * Mf^{-7/6} * Ahat(Mf)
  T pfac, cfac;             // (1 + cos^2 i)/2, cos i
  T af, erad;               // remnant spin and radiated energy (fraction of M)
  T v2c;                    // intermediate amplitude collocation value
};

template <class T>
T amp_ins(const PhenomD<T>& p, const T& Mf) {
  T v = cbrt(Mf);
  T v2 = v * v;
  return 1.0 + p.ampc[0] * v2 + p.ampc[1] * Mf + p.ampc[2] * Mf * v + p.ampc[3] * Mf * v2 + p.ampc[4] * Mf * Mf +
         p.ampc[5] * Mf * Mf * v + p.ampc[6] * Mf * Mf * v2 + p.ampc[7] * Mf * Mf * Mf;
}
template <class T>
T damp_ins(const PhenomD<T>& p, const T& Mf) {
  T v = cbrt(Mf);
  T v2 = v * v;
  return (2.0 / 3.0) * p.ampc[0] / v + p.ampc[1] + (4.0 / 3.0) * p.ampc[2] * v + (5.0 / 3.0) * p.ampc[3] * v2 +
         2.0 * p.ampc[4] * Mf + (7.0 / 3.0) * p.ampc[5] * Mf * v + (8.0 / 3.0) * p.ampc[6] * Mf * v2 +
         3.0 * p.ampc[7] * Mf * Mf;
}
template <class T>
T amp_mrd(const PhenomD<T>& p, const T& Mf) {
  T fdg = p.g3 * p.fDM;
  T df = Mf - p.fRD;
  return p.g1 * fdg / (df * df + fdg * fdg) * exp(-p.g2 * df / fdg);
}
template <class T>
T damp_mrd(const PhenomD<T>& p, const T& Mf) {
  T fdg = p.g3 * p.fDM;
  T df = Mf - p.fRD;
  T den = df * df + fdg * fdg;
  return amp_mrd(p, Mf) * (-p.g2 / fdg - 2.0 * df / den);
}
template <class T>
T amp_int(const PhenomD<T>& p, const T& Mf) {
  return p.dl[0] + Mf * (p.dl[1] + Mf * (p.dl[2] + Mf * (p.dl[3] + Mf * p.dl[4])));
}
template <class T>
T amp_hat(const PhenomD<T>& p, const T& Mf) {
  if (Mf < AMP_F_JOIN_INS) return amp_ins(p, Mf);
  if (Mf >= p.fpeak) return amp_mrd(p, Mf);
  return amp_int(p, Mf);
}

template <class T>
T phi_ins(const PhenomD<T>& p, const T& Mf) {
  T v = cbrt(PI * Mf);
  T logv = log(v);
  T iv = 1.0 / v;
  T iv2 = iv * iv;
  T iv5 = iv2 * iv2 * iv;
  // sum_k (pv_k + pvl_k log v) v^{k-5}
  T s = p.pv[0] * iv5 + p.pv[2] * iv2 * iv + p.pv[3] * iv2 + p.pv[4] * iv + (p.pv[5] + p.pvl[5] * logv) +
        (p.pv[6] + p.pvl[6] * logv) * v + p.pv[7] * v * v;
  T Mf13 = cbrt(Mf);
  T Mf43 = Mf * Mf13, Mf53 = Mf43 * Mf13;
  return s - PI / 4 + (p.s1 * Mf + 0.75 * p.s2 * Mf43 + 0.6 * p.s3 * Mf53 + 0.5 * p.s4 * Mf * Mf) / p.eta;
}
template <class T>
T dphi_ins(const PhenomD<T>& p, const T& Mf) {
  T v = cbrt(PI * Mf);
  T logv = log(v);
  T v2 = v * v, v3 = v2 * v, v4 = v2 * v2, v5 = v4 * v, v6 = v3 * v3, v7 = v6 * v, v8 = v4 * v4;
  T s = 2.0 * p.pv[7] * v7 + (p.pv[6] + p.pvl[6] * (1.0 + logv)) * v6 + p.pvl[5] * v5 - 1.0 * p.pv[4] * v4 -
        2.0 * p.pv[3] * v3 - 3.0 * p.pv[2] * v2 - 5.0 * p.pv[0];
  s = s * (PI / 3.0) / v8;
  T Mf13 = cbrt(Mf);
  return s + (p.s1 + p.s2 * Mf13 + p.s3 * Mf13 * Mf13 + p.s4 * Mf) / p.eta;
}
template <class T>
T phi_int_raw(const PhenomD<T>& p, const T& Mf) {
  return (p.b1 * Mf - p.b3 / (3.0 * Mf * Mf * Mf) + p.b2 * log(Mf)) / p.eta;
}
template <class T>
T dphi_int_raw(const PhenomD<T>& p, const T& Mf) {
  T Mf2 = Mf * Mf;
  return (p.b1 + p.b3 / (Mf2 * Mf2) + p.b2 / Mf) / p.eta;
}
template <class T>
T phi_mrd_raw(const PhenomD<T>& p, const T& Mf) {
  T sq = sqrt(sqrt(Mf));
  return (p.a1 * Mf - p.a2 / Mf + (4.0 / 3.0) * p.a3 * sq * sq * sq + p.a4 * atan((Mf - p.a5 * p.fRD) / p.fDM)) /
         p.eta;
}
template <class T>
T dphi_mrd_raw(const PhenomD<T>& p, const T& Mf) {
  T sq = sqrt(sqrt(Mf));
  T x = Mf - p.a5 * p.fRD;
  return (p.a1 + p.a2 / (Mf * Mf) + p.a3 / sq + p.a4 * p.fDM / (p.fDM * p.fDM + x * x)) / p.eta;
}
template <class T>
T phi_full(const PhenomD<T>& p, const T& Mf) {
  if (Mf < PHI_F_JOIN_INS) return phi_ins(p, Mf);
  if (Mf >= 0.5 * p.fRD) return phi_mrd_raw(p, Mf) + p.C1MRD + p.C2MRD * Mf;
  return phi_int_raw(p, Mf) + p.C1Int + p.C2Int * Mf;
}
template <class T>
T dphi_full(const PhenomD<T>& p, const T& Mf) {
  if (Mf < PHI_F_JOIN_INS) return dphi_ins(p, Mf);
  if (Mf >= 0.5 * p.fRD) return dphi_mrd_raw(p, Mf) + p.C2MRD;
  return dphi_int_raw(p, Mf) + p.C2Int;
}

// Solve a 5x5 system in place (Gaussian elimination, partial pivoting on values).
template <class T>
void solve5(T A[5][5], T b[5], T x[5]) {
  for (int c = 0; c < 5; ++c) {
    int piv = c;
    for (int r = c + 1; r < 5; ++r)
      if (std::fabs(val(A[r][c])) > std::fabs(val(A[piv][c]))) piv = r;
    if (piv != c) {
      for (int j = 0; j < 5; ++j) std::swap(A[c][j], A[piv][j]);
      std::swap(b[c], b[piv]);
    }
    for (int r = c + 1; r < 5; ++r) {
      T m = A[r][c] / A[c][c];
      for (int j = c; j < 5; ++j) A[r][j] = A[r][j] - m * A[c][j];
      b[r] = b[r] - m * b[c];
    }
  }
  for (int r = 4; r >= 0; --r) {
    T s = b[r];
    for (int j = r + 1; j < 5; ++j) s = s - A[r][j] * x[j];
    x[r] = s / A[r][r];
  }
}

// Source parameters (all in one array, the batch parameterisation):
// 0 ln Mc[Msun, detector frame], 1 q=m1/m2>=1, 2 chi1, 3 chi2, 4 ln D_L[Mpc],
// 5 cos(iota), 6 lambda, 7 sin(beta), 8 psi, 9 phi_c, 10 t_c[s]
template <class T>
void phenomd_setup(const T* th, double f_ref, PhenomD<T>& p) {
  T Mc = exp(th[0]);
  T q = th[1];
  T chi1 = th[2], chi2 = th[3];
  T eta = q / ((1.0 + q) * (1.0 + q));
  T Mtot = Mc * pow(eta, -0.6);
  T m1 = q / (1.0 + q), m2 = 1.0 / (1.0 + q);  // fractions of M
  T seta = (q - 1.0) / (q + 1.0);
  p.M_sec = Mtot * MTSUN_SI;
  p.eta = eta;
  p.chi1 = chi1;
  p.chi2 = chi2;
  p.seta = seta;
  T eta2 = eta * eta, eta3 = eta2 * eta;
  // chi_PN (Khan et al. 2016 eq. 2.8)
  T chieff = m1 * chi1 + m2 * chi2;
  T chipn = chieff - 38.0 / 113.0 * eta * (chi1 + chi2);
  T xi = chipn - 1.0;
  // final spin and radiated energy (Husa et al. 2016 fits)
  T s = m1 * m1 * chi1 + m2 * m2 * chi2;
  T s2 = s * s, s3 = s2 * s;
  T af = eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * eta2 -
                13.180949901606242 * eta3 +
                s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) +
                     (0.1014665242971878 - 2.0967746996832157 * eta) * s +
                     (-1.3546806617824356 + 4.108962025369336 * eta) * s2 +
                     (-0.8676969352555539 + 2.064046835273906 * eta) * s3));
  p.af = af;
  T sn = s / (m1 * m1 + m2 * m2);
  T eta4 = eta3 * eta;
  T erad = ((0.055974469826360077 * eta + 0.5809510763115132 * eta2 - 0.9606726679372312 * eta3 +
             3.352411249771192 * eta4) *
            (1.0 + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * sn)) /
           (1.0 + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * sn);
  p.erad = erad;
  // (2,2,0) quasi-normal mode of the remnant (mass 1 - E_rad, spin af): the
  // Kerr frequency M omega = wR - i wI interpolated from the mode table
  T wR, wI;
  qnm_interp(0, af, wR, wI);
  p.fRD = wR / (2.0 * PI) / (1.0 - erad);
  p.fDM = wI / (2.0 * PI) / (1.0 - erad);
  // fits
  T v2c = fit_eval(F_V2, eta, xi);
  p.v2c = v2c;
  p.g1 = fit_eval(F_G1, eta, xi);
  p.g2 = fit_eval(F_G2, eta, xi);
  p.g3 = fit_eval(F_G3, eta, xi);
  p.s1 = fit_eval(F_S1, eta, xi);
  p.s2 = fit_eval(F_S2, eta, xi);
  p.s3 = fit_eval(F_S3, eta, xi);
  p.s4 = fit_eval(F_S4, eta, xi);
  p.b1 = fit_eval(F_B1, eta, xi);
  p.b2 = fit_eval(F_B2, eta, xi);
  p.b3 = fit_eval(F_B3, eta, xi);
  p.a1 = fit_eval(F_A1, eta, xi);
  p.a2 = fit_eval(F_A2, eta, xi);
  p.a3 = fit_eval(F_A3, eta, xi);
  p.a4 = fit_eval(F_A4, eta, xi);
  p.a5 = fit_eval(F_A5, eta, xi);
  // amplitude peak frequency
  if (p.g2 <= 1.0)
    p.fpeak = fabs(p.fRD + (p.fDM * (-1.0 + sqrt(1.0 - p.g2 * p.g2)) * p.g3) / p.g2);
  else
    p.fpeak = fabs(p.fRD + (-p.fDM * p.g3) / p.g2);
  // PN amplitude coefficients of the inspiral ansatz (Khan et al. 2016 appendix B)
  const double pi13 = std::cbrt(PI), pi23 = pi13 * pi13, pi43 = PI * pi13, pi53 = PI * pi23, pi2 = PI * PI;
  T c12 = chi1 * chi1, c22 = chi2 * chi2;
  p.ampc[0] = ((-969.0 + 1804.0 * eta) * pi23) / 672.0;
  p.ampc[1] = ((chi1 * (81.0 * (1.0 + seta) - 44.0 * eta) + chi2 * (81.0 - 81.0 * seta - 44.0 * eta)) * PI) / 48.0;
  p.ampc[2] = ((-27312085.0 - 10287648.0 * c22 - 10287648.0 * c12 * (1.0 + seta) + 10287648.0 * c22 * seta +
                24.0 * (-1975055.0 + 857304.0 * c12 - 994896.0 * chi1 * chi2 + 857304.0 * c22) * eta +
                35371056.0 * eta2) *
               pi43) /
              8128512.0;
  p.ampc[3] = (pi53 * (chi2 * (-285197.0 * (-1.0 + seta) + 4.0 * (-91902.0 + 1579.0 * seta) * eta - 35632.0 * eta2) +
                       chi1 * (285197.0 * (1.0 + seta) - 4.0 * (91902.0 + 1579.0 * seta) * eta - 35632.0 * eta2) +
                       42840.0 * (-1.0 + 4.0 * eta) * PI)) /
              32256.0;
  p.ampc[4] =
      -(pi2 * (-336.0 * (-3248849057.0 + 2943675504.0 * c12 - 3339284256.0 * chi1 * chi2 + 2943675504.0 * c22) * eta2 -
               324322727232.0 * eta3 -
               7.0 * (-177520268561.0 + 107414046432.0 * c22 + 107414046432.0 * c12 * (1.0 + seta) -
                      107414046432.0 * c22 * seta + 11087290368.0 * (chi1 + chi2 + chi1 * seta - chi2 * seta) * PI) +
               12.0 * eta *
                   (-545384828789.0 - 176491177632.0 * chi1 * chi2 + 202603761360.0 * c22 +
                    77616.0 * c12 * (2610335.0 + 995766.0 * seta) - 77287373856.0 * c22 * seta +
                    5841690624.0 * (chi1 + chi2) * PI + 21384760320.0 * pi2))) /
      60085960704.0;
  // the calibrated inspiral terms rho1 Mf^{7/3} + rho2 Mf^{8/3} + rho3 Mf^3 (Khan et al. 2016 eq. 29)
  p.ampc[5] = fit_eval(F_R1, eta, xi);
  p.ampc[6] = fit_eval(F_R2, eta, xi);
  p.ampc[7] = fit_eval(F_R3, eta, xi);
  // intermediate amplitude: match value/derivative at 0.014 and fpeak, value v2 in between
  {
    T f1 = T(AMP_F_JOIN_INS), f3 = p.fpeak, f2 = 0.5 * (f1 + f3);
    T A[5][5], b[5];
    T fs[3] = {f1, f2, f3};
    for (int r = 0; r < 3; ++r) {
      T pw = T(1.0);
      for (int j = 0; j < 5; ++j) { A[r][j] = pw; pw = pw * fs[r]; }
    }
    // derivative rows
    T fd[2] = {f1, f3};
    for (int r = 0; r < 2; ++r) {
      A[3 + r][0] = T(0.0);
      A[3 + r][1] = T(1.0);
      A[3 + r][2] = 2.0 * fd[r];
      A[3 + r][3] = 3.0 * fd[r] * fd[r];
      A[3 + r][4] = 4.0 * fd[r] * fd[r] * fd[r];
    }
    b[0] = amp_ins(p, f1);
    b[1] = v2c;
    b[2] = amp_mrd(p, f3);
    b[3] = damp_ins(p, f1);
    b[4] = damp_mrd(p, f3);
    solve5(A, b, p.dl);
  }
  // TaylorF2 aligned-spin phasing without the 3PN spin-spin term
  {
    T SL = m1 * m1 * chi1 + m2 * m2 * chi2;
    T dSL = seta * (m2 * chi2 - m1 * chi1);
    T pn_sigma = eta * (721.0 / 48.0 * chi1 * chi2 - 247.0 / 48.0 * chi1 * chi2) +
                 (720.0 - 1.0) / 96.0 * m1 * m1 * c12 + (720.0 - 1.0) / 96.0 * m2 * m2 * c22 -
                 (240.0 - 7.0) / 96.0 * m1 * m1 * c12 - (240.0 - 7.0) / 96.0 * m2 * m2 * c22;
    T pn_gamma = (554345.0 / 1134.0 + 110.0 * eta / 9.0) * SL + (13915.0 / 84.0 - 10.0 * eta / 3.0) * dSL;
    T pfaN = 3.0 / (128.0 * eta);
    T v[8], vl[8];
    for (int i = 0; i < 8; ++i) { v[i] = T(0.0); vl[i] = T(0.0); }
    v[0] = T(1.0);
    v[2] = 5.0 * (743.0 / 84.0 + 11.0 * eta) / 9.0;
    v[3] = -16.0 * PI + 188.0 * SL / 3.0 + 25.0 * dSL;
    v[4] = 5.0 * (3058.673 / 7.056 + 5429.0 / 7.0 * eta + 617.0 * eta2) / 72.0 - 10.0 * pn_sigma;
    v[5] = 5.0 / 9.0 * (7729.0 / 84.0 - 13.0 * eta) * PI - pn_gamma;
    vl[5] = 5.0 / 3.0 * (7729.0 / 84.0 - 13.0 * eta) * PI - 3.0 * pn_gamma;
    v[6] = (11583.231236531 / 4.694215680 - 640.0 / 3.0 * PI * PI - 6848.0 / 21.0 * EULER_GAMMA) +
           eta * (-15737.765635 / 3.048192 + 2255.0 / 12.0 * PI * PI) + eta2 * 76055.0 / 1728.0 -
           eta3 * 127825.0 / 1296.0 + (-6848.0 / 21.0) * std::log(4.0) + PI * (3760.0 * SL + 1490.0 * dSL) / 3.0;
    vl[6] = T(-6848.0 / 21.0);
    v[7] = PI * (77096675.0 / 254016.0 + 378515.0 / 1512.0 * eta - 74045.0 / 756.0 * eta2) +
           (-8980424995.0 / 762048.0 + 6586595.0 * eta / 756.0 - 305.0 * eta2 / 36.0) * SL -
           (170978035.0 / 48384.0 - 2876425.0 * eta / 672.0 - 4735.0 * eta2 / 144.0) * dSL;
    for (int i = 0; i < 8; ++i) { p.pv[i] = v[i] * pfaN; p.pvl[i] = vl[i] * pfaN; }
  }
  // C1 continuity of the phase at 0.018 and at fRD/2
  {
    T f1 = T(PHI_F_JOIN_INS);
    p.C2Int = dphi_ins(p, f1) - dphi_int_raw(p, f1);
    p.C1Int = phi_ins(p, f1) - phi_int_raw(p, f1) - p.C2Int * f1;
    T f2 = 0.5 * p.fRD;
    T phi_int_f2 = phi_int_raw(p, f2) + p.C1Int + p.C2Int * f2;
    T dphi_int_f2 = dphi_int_raw(p, f2) + p.C2Int;
    p.C2MRD = dphi_int_f2 - dphi_mrd_raw(p, f2);
    p.C1MRD = phi_int_f2 - phi_mrd_raw(p, f2) - p.C2MRD * f2;
  }
  // time and phase alignment: t(fpeak) = 0, Psi(f_ref) = -2 phi_c
  p.t0 = dphi_full(p, p.fpeak);
  p.MfRef = p.M_sec * f_ref;
  p.phi_shift = phi_full(p, p.MfRef) + 2.0 * th[9];
  // overall amplitude: 2 sqrt(5/(64 pi)) M^2/D_L * sqrt(2 eta/3) pi^{-1/6}
  T DL_m = exp(th[4]) * (1.0e6 * PC_SI);
  T amp0 = 2.0 * std::sqrt(5.0 / (64.0 * PI)) * (Mtot * MRSUN_SI) * (Mtot * MTSUN_SI) / DL_m;
  p.amp_scale = amp0 * sqrt(2.0 * eta / 3.0) / std::pow(PI, 1.0 / 6.0);
  p.pfac = 0.5 * (1.0 + th[5] * th[5]);
  p.cfac = th[5];
}

// Plus/cross polarisations and t(f) of the (2,2) waveform at frequency f [Hz];
// zero above f_cut_hz.  Returns false when the bin is cut.
template <class T>
bool phenomd_eval(const PhenomD<T>& p, double f, double f_cut_hz, Cx<T>& hp, Cx<T>& hc, T& tf,
                  T* amp_out = nullptr, T* psi_out = nullptr) {
  T Mf = p.M_sec * f;
  if (f > f_cut_hz || Mf > MF_CUT) {
    hp = Cx<T>{T(0.0), T(0.0)};
    hc = Cx<T>{T(0.0), T(0.0)};
    tf = T(0.0);
    return false;
  }
  T v = cbrt(Mf);
  // Mf^{7/6} = Mf * Mf^{1/6}; Mf^{1/6} = sqrt(Mf^{1/3})
  T amp = p.amp_scale / (Mf * sqrt(v)) * amp_hat(p, Mf);
  T psi = phi_full(p, Mf) - p.t0 * (Mf - p.MfRef) - p.phi_shift;
  tf = p.M_sec / (2.0 * PI) * (dphi_full(p, Mf) - p.t0);
  if (amp_out) *amp_out = amp;
  if (psi_out) *psi_out = psi;
  T c = cos(psi), s = sin(psi);
  // h22 = amp e^{-i psi}; hp = pfac h22, hc = -i cfac h22
  hp = Cx<T>{p.pfac * amp * c, -(p.pfac * amp * s)};
  hc = Cx<T>{-(p.cfac * amp * s), -(p.cfac * amp * c)};
  return true;
}

// ----------------------------------------------------------------- IMRPhenomHM
// The higher-multipole model of London et al. 2018 (arXiv:1708.00404), built
// from the (2,2) IMRPhenomD as the paper does:
//  * each mode's frequency maps onto the (2,2) frequency f22: f22 = 2 f / m
//    in the inspiral (same orbital frequency), f22 = Rholm f in the ringdown
//    (Rholm = fRD22 / fRD_lm, so the mode's ringdown sits at its own Kerr QNM
//    frequency); between the corners the phase map is linear (the paper's),
//    the amplitude map the cubic Hermite blend of the two lines (value and
//    slope matched, so that the amplitude stays C1); the amplitude map's
//    corners are the (2,2) amplitude joins Mf = 0.014 and f_peak, the phase
//    map's the (2,2) phase joins Mf = 0.018 and fRD22 / 2;
//  * amplitude A_lm(f) = beta_lm A22(f22): beta_lm the ratio of the
//    post-Newtonian mode amplitudes |H_lm| / |H_22| sqrt(2/m) at the
//    orbital velocity v = (2 pi M f_b / m)^{1/3} (leading order with the 1PN
//    corrections of the l = m modes and the leading spin term of (2,1);
//    Blanchet, Living Rev. Rel. 17, 2 (2014) eq. 327; Arun et al. 2009),
//    f_b = f below the amplitude map's inspiral corner f_i and
//    f_i (2 - exp(1 - f/f_i)) above it (C1, saturating at 2 f_i); A22 the
//    PhenomD amplitude whose merger-ringdown Lorentzian width is the mode's,
//    in mapped frequency Rholm fDM_lm (intermediate collocation re-solved);
//  * phase Psi_lm(f) = (m/2) Psi22(2 f / m) in the inspiral,
//    (1/a) Psi22(a f + b) + c0 + c1 f between the corners and
//    (1/Rholm) Psi22^MRD(Rholm f) + c0' + c1' f in the ringdown, with the
//    damping of the arctangent the mode's (Rholm fDM_lm in mapped
//    frequency) and c0, c1, c0', c1' making Psi_lm C1; plus the constant
//    phase of H_lm (k quarter turns).  t_lm(f) = dPsi_lm/df / (2 pi).
//  * polarisations: hp = sum P_lm h_lm, hc = i sum C_lm h_lm with
//    P_lm = [(-1)^l Y_{l,-m} + Y_lm] / (2 N), C_lm = [(-1)^l Y_{l,-m} - Y_lm] / (2 N),
//    Y the s = -2 spherical harmonics at azimuth 0 (Wigner d^l_{m,2}) and
//    N = sqrt(5 / (16 pi)), so that (2,2) gives PhenomD's (1 + cos^2 i)/2, -cos i.
// Modes (in this order): (2,2), (2,1), (3,3), (3,2), (4,4), (4,3) (also the
// order of the quasi-normal-mode table).
constexpr int HM_MODES = 6;
static const int kHMlm[HM_MODES][2] = {{2, 2}, {2, 1}, {3, 3}, {3, 2}, {4, 4}, {4, 3}};

static double factorial(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}

// s = -2 spin-weighted spherical harmonic at azimuth 0 from cos(iota):
// sqrt((2l+1)/(4 pi)) d^l_{m,2}(iota)
template <class T>
T sylm_m2(int l, int m, const T& cosi) {
  T ch = sqrt(0.5 * (1.0 + cosi)), sh = sqrt(0.5 * (1.0 - cosi));
  T sum = T(0.0);
  for (int k = 0; k <= l + m; ++k) {
    if (l + m - k < 0 || l - 2 - k < 0 || k + 2 - m < 0) continue;
    const double c = ((k & 1) ? -1.0 : 1.0) *
                     std::sqrt(factorial(l + m) * factorial(l - m) * factorial(l + 2) * factorial(l - 2)) /
                     (factorial(l + m - k) * factorial(l - 2 - k) * factorial(k) * factorial(k + 2 - m));
    T term = T(c);
    for (int e = 0; e < 2 * l + m - 2 * k - 2; ++e) term = term * ch;
    for (int e = 0; e < 2 * k + 2 - m; ++e) term = term * sh;
    sum = sum + term;
  }
  return std::sqrt((2.0 * l + 1.0) / (4.0 * PI)) * sum;
}

// Signed post-Newtonian amplitude ratio beta_lm(v) and the quarter turns of
// H_lm's phase (H_lm = i^k |.|).
template <class T>
T hm_pn_ratio(int l, int m, const T& v, const T& eta, const T& dlt, const T& chis, const T& chia, int* kq) {
  T v2 = v * v;
  T h22 = 1.0 + v2 * (-107.0 / 42.0 + 55.0 / 42.0 * eta) + 2.0 * PI * v2 * v;
  T r;
  if (l == 2 && m == 2) { *kq = 0; return T(1.0); }
  if (l == 2 && m == 1) {
    *kq = 1;
    r = (1.0 / 3.0) * (dlt * v * (1.0 + v2 * (-17.0 / 28.0 + 5.0 / 7.0 * eta)) - 1.5 * (chia + dlt * chis) * v2);
  } else if (l == 3 && m == 3) {
    *kq = 3;
    r = 0.75 * std::sqrt(15.0 / 14.0) * dlt * v * (1.0 + v2 * (-4.0 + 2.0 * eta));
  } else if (l == 3 && m == 2) {
    *kq = 0;
    r = (1.0 / 3.0) * std::sqrt(5.0 / 7.0) * v2 * (1.0 - 3.0 * eta);
  } else if (l == 4 && m == 4) {
    *kq = 2;
    r = (8.0 / 9.0) * std::sqrt(5.0 / 7.0) * v2 * (1.0 - 3.0 * eta);
  } else {  // (4,3)
    *kq = 3;
    r = 9.0 / (4.0 * std::sqrt(70.0)) * dlt * v2 * v * (1.0 - 2.0 * eta);
  }
  return r / h22 * std::sqrt(2.0 / m);
}

template <class T>
struct PhenomHMMode {
  int l, m, kq;
  T P, C;                          // polarisation factors
  T Rholm, fRD, fDMeff, g3fDMeff;  // fRD: the mode's ringdown frequency (Mf)
  T fpeak, dl[5];                  // amplitude in mapped frequency: peak, intermediate polynomial
  T fiA, frA;                      // amplitude map corners (Mf)
  T fiP, frP, aP, bP;              // phase map
  T cI0, cI1, cR0, cR1;            // C1 constants of the phase
};

template <class T>
struct PhenomHM {
  PhenomD<T> d;
  PhenomHMMode<T> md[HM_MODES];
  T eta, dlt, chis, chia;
  T fRD_max;  // largest ringdown frequency of the modes (Mf)
};

// the amplitude's frequency map: 2 f / m below fiA, Rholm f above frA, the
// cubic Hermite blend of the two (values and slopes) between
template <class T>
T hm_amp_map(const PhenomHMMode<T>& md, const T& Mf) {
  if (md.l == 2 && md.m == 2) return Mf;  // the identity for (2,2), exactly
  if (Mf <= md.fiA) return (2.0 / md.m) * Mf;
  if (Mf >= md.frA) return md.Rholm * Mf;
  const T h = md.frA - md.fiA, s = (Mf - md.fiA) / h;
  const T s2 = s * s, s3 = s2 * s;
  return (2.0 * s3 - 3.0 * s2 + 1.0) * ((2.0 / md.m) * md.fiA) + (s3 - 2.0 * s2 + s) * (h * (2.0 / md.m)) +
         (3.0 * s2 - 2.0 * s3) * (md.Rholm * md.frA) + (s3 - s2) * (h * md.Rholm);
}

// mapped (2,2) amplitude hat with the mode's merger-ringdown width
template <class T>
T hm_amp_hat(const PhenomHM<T>& h, const PhenomHMMode<T>& md, const T& Mf22) {
  const PhenomD<T>& p = h.d;
  if (Mf22 < AMP_F_JOIN_INS) return amp_ins(p, Mf22);
  if (Mf22 >= md.fpeak) {
    T x = Mf22 - p.fRD;
    return p.g1 * md.g3fDMeff / (x * x + md.g3fDMeff * md.g3fDMeff) * exp(-p.g2 * x / md.g3fDMeff);
  }
  return md.dl[0] + Mf22 * (md.dl[1] + Mf22 * (md.dl[2] + Mf22 * (md.dl[3] + Mf22 * md.dl[4])));
}

// (2,2) phase and its Mf-derivative (aligned: Psi = Phi - t0 (Mf - MfRef) - shift)
template <class T>
void hm_psi22(const PhenomD<T>& p, const T& Mf, T& psi, T& dpsi) {
  psi = phi_full(p, Mf) - p.t0 * (Mf - p.MfRef) - p.phi_shift;
  dpsi = dphi_full(p, Mf) - p.t0;
}
// the (2,2) merger-ringdown phase ansatz with damping fdm
template <class T>
void hm_psi22_mrd(const PhenomD<T>& p, const T& fdm, const T& Mf, T& psi, T& dpsi) {
  T sq = sqrt(sqrt(Mf));
  T x = Mf - p.a5 * p.fRD;
  psi = (p.a1 * Mf - p.a2 / Mf + (4.0 / 3.0) * p.a3 * sq * sq * sq + p.a4 * atan(x / fdm)) / p.eta + p.C1MRD +
        p.C2MRD * Mf - p.t0 * (Mf - p.MfRef) - p.phi_shift;
  dpsi = (p.a1 + p.a2 / (Mf * Mf) + p.a3 / sq + p.a4 * fdm / (fdm * fdm + x * x)) / p.eta + p.C2MRD - p.t0;
}

// Psi_lm and dPsi_lm/dMf without the constant quarter turns; region by Mf
template <class T>
void hm_phase(const PhenomHM<T>& h, const PhenomHMMode<T>& md, const T& Mf, T& psi, T& dpsi) {
  if (Mf < md.fiP) {
    hm_psi22(h.d, (2.0 / md.m) * Mf, psi, dpsi);
    psi = (0.5 * md.m) * psi;
  } else if (Mf < md.frP) {
    hm_psi22(h.d, md.aP * Mf + md.bP, psi, dpsi);
    psi = psi / md.aP + md.cI0 + md.cI1 * Mf;
    dpsi = dpsi + md.cI1;
  } else {
    hm_psi22_mrd(h.d, md.fDMeff, md.Rholm * Mf, psi, dpsi);
    psi = psi / md.Rholm + md.cR0 + md.cR1 * Mf;
    dpsi = dpsi + md.cR1;
  }
}

template <class T>
void phenomhm_setup(const T* th, double f_ref, PhenomHM<T>& h) {
  PhenomD<T>& p = h.d;
  phenomd_setup(th, f_ref, p);
  T q = th[1];
  h.eta = p.eta;
  h.dlt = (q - 1.0) / (q + 1.0);
  h.chis = 0.5 * (th[2] + th[3]);
  h.chia = 0.5 * (th[2] - th[3]);
  const double nrm = 2.0 * std::sqrt(5.0 / (64.0 * PI));
  h.fRD_max = p.fRD;
  for (int k = 0; k < HM_MODES; ++k) {
    PhenomHMMode<T>& md = h.md[k];
    md.l = kHMlm[k][0];
    md.m = kHMlm[k][1];
    const int l = md.l, m = md.m;
    T Yp = sylm_m2(l, m, th[5]), Ym = sylm_m2(l, -m, th[5]);
    const double sg = (l & 1) ? -1.0 : 1.0;
    md.P = (sg * Ym + Yp) / (2.0 * nrm);
    md.C = (sg * Ym - Yp) / (2.0 * nrm);
    // the mode's Kerr quasi-normal mode
    T wR, wI;
    qnm_interp(k, p.af, wR, wI);
    md.fRD = wR / (2.0 * PI) / (1.0 - p.erad);
    T fDMlm = wI / (2.0 * PI) / (1.0 - p.erad);
    if (val(md.fRD) > val(h.fRD_max)) h.fRD_max = md.fRD;
    md.Rholm = p.fRD / md.fRD;
    md.fDMeff = md.Rholm * fDMlm;
    md.g3fDMeff = p.g3 * md.fDMeff;
    if (p.g2 <= 1.0)
      md.fpeak = fabs(p.fRD + (md.fDMeff * (-1.0 + sqrt(1.0 - p.g2 * p.g2)) * p.g3) / p.g2);
    else
      md.fpeak = fabs(p.fRD + (-md.fDMeff * p.g3) / p.g2);
    // intermediate amplitude with the mode's merger-ringdown: value/derivative at 0.014 and fpeak, v2 midway
    {
      T f1 = T(AMP_F_JOIN_INS), f3 = md.fpeak, f2 = 0.5 * (f1 + f3);
      T A[5][5], b[5];
      T fs[3] = {f1, f2, f3};
      for (int r = 0; r < 3; ++r) {
        T pw = T(1.0);
        for (int j = 0; j < 5; ++j) { A[r][j] = pw; pw = pw * fs[r]; }
      }
      T fd[2] = {f1, f3};
      for (int r = 0; r < 2; ++r) {
        A[3 + r][0] = T(0.0);
        A[3 + r][1] = T(1.0);
        A[3 + r][2] = 2.0 * fd[r];
        A[3 + r][3] = 3.0 * fd[r] * fd[r];
        A[3 + r][4] = 4.0 * fd[r] * fd[r] * fd[r];
      }
      T x3 = f3 - p.fRD, den = x3 * x3 + md.g3fDMeff * md.g3fDMeff;
      T Amrd = p.g1 * md.g3fDMeff / den * exp(-p.g2 * x3 / md.g3fDMeff);
      b[0] = amp_ins(p, f1);
      b[1] = p.v2c;
      b[2] = Amrd;
      b[3] = damp_ins(p, f1);
      b[4] = Amrd * (-p.g2 / md.g3fDMeff - 2.0 * x3 / den);
      solve5(A, b, md.dl);
    }
    // maps: corners at the (2,2) joins, inspiral slope 2/m, ringdown slope Rholm
    md.fiA = (0.5 * m) * AMP_F_JOIN_INS;
    md.frA = md.fpeak / md.Rholm;
    int kq;
    hm_pn_ratio(l, m, T(0.1), h.eta, h.dlt, h.chis, h.chia, &kq);
    md.kq = kq;
    md.fiP = (0.5 * m) * PHI_F_JOIN_INS;
    md.frP = (0.5 * p.fRD) / md.Rholm;
    md.aP = (0.5 * p.fRD - PHI_F_JOIN_INS) / (md.frP - md.fiP);
    md.bP = PHI_F_JOIN_INS - md.aP * md.fiP;
    // C1 matching of the phase at fiP and frP
    md.cI0 = md.cI1 = md.cR0 = md.cR1 = T(0.0);
    T v1, d1, v2_, d2;
    hm_psi22(p, (2.0 / m) * md.fiP, v1, d1);
    v1 = (0.5 * m) * v1;
    hm_psi22(p, md.aP * md.fiP + md.bP, v2_, d2);
    v2_ = v2_ / md.aP;
    md.cI1 = d1 - d2;
    md.cI0 = v1 - v2_ - md.cI1 * md.fiP;
    T v3, d3;
    hm_psi22(p, md.aP * md.frP + md.bP, v2_, d2);
    v2_ = v2_ / md.aP + md.cI0 + md.cI1 * md.frP;
    d2 = d2 + md.cI1;
    hm_psi22_mrd(p, md.fDMeff, md.Rholm * md.frP, v3, d3);
    v3 = v3 / md.Rholm;
    md.cR1 = d2 - d3;
    md.cR0 = v2_ - v3 - md.cR1 * md.frP;
  }
}

// Mode k: amplitude, phase (including the quarter turns) and t(f) at f [Hz];
// false where the mode is zero (above f_cut_hz or above mapped Mf = 0.2).
template <class T>
bool phenomhm_mode(const PhenomHM<T>& h, int k, double f, double f_cut_hz, T& amp, T& psi, T& tf) {
  const PhenomD<T>& p = h.d;
  const PhenomHMMode<T>& md = h.md[k];
  T Mf = p.M_sec * f;
  T f22A = hm_amp_map(md, Mf);
  if (f > f_cut_hz || f22A > MF_CUT) {
    amp = T(0.0);
    psi = T(0.0);
    tf = T(0.0);
    return false;
  }
  int kq;
  const T fb = (Mf <= md.fiA) ? Mf : md.fiA * (2.0 - exp(1.0 - Mf / md.fiA));
  const T beta = hm_pn_ratio(md.l, md.m, cbrt(2.0 * PI * fb / md.m), h.eta, h.dlt, h.chis, h.chia, &kq);
  T v = cbrt(f22A);
  amp = beta * (p.amp_scale / (f22A * sqrt(v)) * hm_amp_hat(h, md, f22A));
  T dpsi;
  hm_phase(h, md, Mf, psi, dpsi);
  psi = psi + md.kq * (0.5 * PI);
  tf = p.M_sec / (2.0 * PI) * dpsi;
  return true;
}

// ----------------------------------------------------------------- batch lnL
struct OracleDet {
  OrbitDesc orbit;
  int32_t gen20;
  int32_t pad;
  const double* data;     // (3, nbins) complex, interleaved re/im, A/E/T
  const double* psd;      // (3, nbins)
};

struct OraclePlan {
  int64_t nbins;
  int64_t k0;        // index of the first bin in the rfft grid
  double f_step;     // rfft spacing 1/(Nt dt)
  double df;         // likelihood weight 1/T (tdi.py:130)
  double f_ref;
  double cut_factor; // per-sample cutoff = cut_factor * fRD (0: PhenomD Mf=0.2 cut only)
  int32_t n_det;
  int32_t chan_mask; // bit c set: channel c (A=0, E=1, T=2) enters the likelihood
  const OracleDet* dets;
  int32_t approximant;  // 0: IMRPhenomD (2,2); 1: IMRPhenomHM (six modes)
  int32_t pad;
};

template <class T>
double sample_cut_hz(const PhenomD<T>& p, double cut_factor, double fmax) {
  double fc = fmax;
  if (cut_factor > 0.0) fc = std::min(fmax, cut_factor * val(p.fRD) / val(p.M_sec));
  return fc;
}

// The plan's waveform: IMRPhenomD, or IMRPhenomHM with its six modes.
template <class T>
struct OracleWave {
  int approx;
  PhenomHM<T> hm;  // hm.d is the PhenomD of either approximant
};

template <class T>
void wave_setup(int approx, const T* th, double f_ref, OracleWave<T>& w) {
  w.approx = approx;
  if (approx == 1)
    phenomhm_setup(th, f_ref, w.hm);
  else
    phenomd_setup(th, f_ref, w.hm.d);
}

template <class T>
double wave_cut_hz(const OracleWave<T>& w, double cut_factor, double fmax) {
  double fc = fmax;
  const double frd = val(w.approx == 1 ? w.hm.fRD_max : w.hm.d.fRD);
  if (cut_factor > 0.0) fc = std::min(fmax, cut_factor * frd / val(w.hm.d.M_sec));
  return fc;
}

// The waveform container's modes at f: hp, hc, tf per mode; returns the
// number of modes (zero containers for modes that are cut) and sets *live.
template <class T>
int wave_eval(const OracleWave<T>& w, double f, double fcut, Cx<T>* hp, Cx<T>* hc, T* tf, bool* live) {
  if (w.approx != 1) {
    *live = phenomd_eval(w.hm.d, f, fcut, hp[0], hc[0], tf[0]);
    return 1;
  }
  *live = false;
  for (int k = 0; k < HM_MODES; ++k) {
    T amp, psi;
    if (phenomhm_mode(w.hm, k, f, fcut, amp, psi, tf[k])) {
      *live = true;
      const T c = cos(psi), sn = sin(psi);
      const PhenomHMMode<T>& md = w.hm.md[k];
      // h_lm = amp e^{-i psi}; hp = P h_lm, hc = i C h_lm
      hp[k] = Cx<T>{md.P * amp * c, -(md.P * amp * sn)};
      hc[k] = Cx<T>{md.C * amp * sn, md.C * amp * c};
    } else {
      hp[k] = Cx<T>{T(0.0), T(0.0)};
      hc[k] = Cx<T>{T(0.0), T(0.0)};
    }
  }
  return HM_MODES;
}

template <class T>
T lnl_one(const OraclePlan& pl, const T* th) {
  OracleWave<T> wv;
  wave_setup(pl.approximant, th, pl.f_ref, wv);
  T sb = th[7];
  T cb = sqrt((1.0 - sb) * (1.0 + sb));
  T P[3][3], X[3][3], k[3];
  polarization(th[6], sb, cb, th[8], P, X, k);
  double fmax = double(pl.k0 + pl.nbins - 1) * pl.f_step + 1.0;
  double fcut = wave_cut_hz(wv, pl.cut_factor, fmax);
  // Neumaier-compensated sums in FP64
  T acc = T(0.0);
  double comp = 0.0;
  for (int64_t i = 0; i < pl.nbins; ++i) {
    double f = double(pl.k0 + i) * pl.f_step;
    Cx<T> hp[HM_MODES], hc[HM_MODES];
    T tf[HM_MODES];
    bool live;
    const int nm = wave_eval(wv, f, fcut, hp, hc, tf, &live);
    T bin = T(0.0);
    for (int d = 0; d < pl.n_det; ++d) {
      const OracleDet& det = pl.dets[d];
      Cx<T> h[3] = {{T(0.0), T(0.0)}, {T(0.0), T(0.0)}, {T(0.0), T(0.0)}};
      if (live) {
        Cx<T> L[6];
        response_at_f(det.orbit, f, nm, hp, hc, tf, th[10], P, X, k, L);
        tdi_at_f(f, det.orbit.arm_sec, det.gen20, 1, L, h);
      }
      for (int c = 0; c < 3; ++c) {
        if (!((pl.chan_mask >> c) & 1)) continue;
        double dre = det.data[2 * (c * pl.nbins + i)], dim = det.data[2 * (c * pl.nbins + i) + 1];
        T rre = dre - h[c].re, rim = dim - h[c].im;
        bin = bin + (rre * rre + rim * rim) / det.psd[c * pl.nbins + i];
      }
    }
    // compensated accumulation on the value; derivatives accumulate plainly
    double a = val(acc), b = val(bin);
    double s = a + b;
    comp += (std::fabs(a) >= std::fabs(b)) ? (a - s) + b : (b - s) + a;
    acc = acc + bin;
  }
  acc = acc + comp;
  return -2.0 * pl.df * acc;
}

// Fisher matrix at one parameter set, fisher.py:27-162:
// F_ij = 4 df Re sum_{det, c, f} conj(dh_i) dh_j / S_c(f) over the channels of
// the mask and the live bins (the model is zero above the sample's cut, so
// its derivatives are too); derivatives by forward-mode dual numbers.
void fisher_one(const OraclePlan& pl, const double* t, double* F) {
  using D11 = Dual<11>;
  D11 th[11];
  for (int j = 0; j < 11; ++j) {
    th[j] = D11(t[j]);
    th[j].d[j] = 1.0;
  }
  OracleWave<D11> wv;
  wave_setup(pl.approximant, th, pl.f_ref, wv);
  D11 sb = th[7];
  D11 cb = sqrt((1.0 - sb) * (1.0 + sb));
  D11 P[3][3], X[3][3], k[3];
  polarization(th[6], sb, cb, th[8], P, X, k);
  double fmax = double(pl.k0 + pl.nbins - 1) * pl.f_step + 1.0;
  double fcut = wave_cut_hz(wv, pl.cut_factor, fmax);
  double acc[11][11] = {};
  for (int64_t i = 0; i < pl.nbins; ++i) {
    double f = double(pl.k0 + i) * pl.f_step;
    Cx<D11> hp[HM_MODES], hc[HM_MODES];
    D11 tf[HM_MODES];
    bool live;
    const int nm = wave_eval(wv, f, fcut, hp, hc, tf, &live);
    if (!live) continue;
    for (int d = 0; d < pl.n_det; ++d) {
      const OracleDet& det = pl.dets[d];
      Cx<D11> L[6], h[3];
      response_at_f(det.orbit, f, nm, hp, hc, tf, th[10], P, X, k, L);
      tdi_at_f(f, det.orbit.arm_sec, det.gen20, 1, L, h);
      for (int c = 0; c < 3; ++c) {
        if (!((pl.chan_mask >> c) & 1)) continue;
        const double w = 1.0 / det.psd[c * pl.nbins + i];
        for (int a = 0; a < 11; ++a)
          for (int b = a; b < 11; ++b) acc[a][b] += w * (h[c].re.d[a] * h[c].re.d[b] + h[c].im.d[a] * h[c].im.d[b]);
      }
    }
  }
  for (int a = 0; a < 11; ++a)
    for (int b = a; b < 11; ++b) F[11 * a + b] = F[11 * b + a] = 4.0 * pl.df * acc[a][b];
}

}  // namespace orc

using namespace orc;

extern "C" {

int oracle_orbit(const OrbitDesc* o, const double* t, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    double nn[3][3], xx[3][3];
    constellation<double>(*o, t[i], nn, xx);
    for (int a = 0; a < 3; ++a)
      for (int j = 0; j < 3; ++j) {
        out[i * 18 + a * 3 + j] = nn[a][j];
        out[i * 18 + 9 + a * 3 + j] = xx[a][j];
      }
  }
  return 0;
}

int oracle_polarization(double lam, double beta, double psi, double* plus9, double* cross9, double* k3) {
  double P[3][3], X[3][3], k[3];
  polarization<double>(lam, std::sin(beta), std::cos(beta), psi, P, X, k);
  for (int i = 0; i < 3; ++i) {
    k3[i] = k[i];
    for (int j = 0; j < 3; ++j) { plus9[3 * i + j] = P[i][j]; cross9[3 * i + j] = X[i][j]; }
  }
  return 0;
}

// hp, hc: (nmodes, n) complex interleaved; tf: (nmodes, n); links out: (6, n) complex
int oracle_response_links(const OrbitDesc* o, const double* f, int64_t n, int nmodes, const double* hp,
                          const double* hc, const double* tf, double lam, double beta, double psi, double tc,
                          double* links) {
  double P[3][3], X[3][3], k[3];
  polarization<double>(lam, std::sin(beta), std::cos(beta), psi, P, X, k);
  std::vector<Cx<double>> mp(nmodes), mc(nmodes);
  std::vector<double> mt(nmodes);
  for (int64_t i = 0; i < n; ++i) {
    for (int m = 0; m < nmodes; ++m) {
      mp[m] = Cx<double>{hp[2 * (m * n + i)], hp[2 * (m * n + i) + 1]};
      mc[m] = Cx<double>{hc[2 * (m * n + i)], hc[2 * (m * n + i) + 1]};
      mt[m] = tf[m * n + i];
    }
    Cx<double> L[6];
    response_at_f<double>(*o, f[i], nmodes, mp.data(), mc.data(), mt.data(), tc, P, X, k, L);
    for (int l = 0; l < 6; ++l) { links[2 * (l * n + i)] = L[l].re; links[2 * (l * n + i) + 1] = L[l].im; }
  }
  return 0;
}

int oracle_tdi(const double* f, int64_t n, double arm, int gen20, int orth, const double* links, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    Cx<double> L[6], C[3];
    for (int l = 0; l < 6; ++l) L[l] = Cx<double>{links[2 * (l * n + i)], links[2 * (l * n + i) + 1]};
    tdi_at_f<double>(f[i], arm, gen20, orth, L, C);
    for (int c = 0; c < 3; ++c) { out[2 * (c * n + i)] = C[c].re; out[2 * (c * n + i) + 1] = C[c].im; }
  }
  return 0;
}

// likelihood_ti.py:58-68: -2 df sum_i sum_c |d - h|^2 / S, sequential compensated sum
double oracle_whittle(const double* d, const double* h, const double* S, int nchan, int64_t n, double df) {
  double acc = 0.0, comp = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double ip = 0.0;
    for (int c = 0; c < nchan; ++c) {
      double rr = d[2 * (c * n + i)] - h[2 * (c * n + i)];
      double ri = d[2 * (c * n + i) + 1] - h[2 * (c * n + i) + 1];
      ip += (rr * rr + ri * ri) / S[c * n + i];
    }
    double s = acc + ip;
    comp += (std::fabs(acc) >= std::fabs(ip)) ? (acc - s) + ip : (ip - s) + acc;
    acc = s;
  }
  return -2.0 * df * (acc + comp);
}

// PhenomD container on arbitrary frequencies; hp, hc complex interleaved.
int oracle_phenomd(const double* th, const double* f, int64_t n, double f_ref, double f_cut_hz, double* hp, double* hc,
                   double* tf, double* info, double* amp_psi) {
  PhenomD<double> p;
  phenomd_setup<double>(th, f_ref, p);
  for (int64_t i = 0; i < n; ++i) {
    Cx<double> a, b;
    double t, am = 0.0, ps = 0.0;
    phenomd_eval<double>(p, f[i], f_cut_hz, a, b, t, &am, &ps);
    if (amp_psi) { amp_psi[2 * i] = am; amp_psi[2 * i + 1] = ps; }
    hp[2 * i] = a.re; hp[2 * i + 1] = a.im;
    hc[2 * i] = b.re; hc[2 * i + 1] = b.im;
    tf[i] = t;
  }
  if (info) {
    info[0] = p.M_sec; info[1] = p.fRD; info[2] = p.fDM; info[3] = p.fpeak; info[4] = p.t0;
    info[5] = p.eta; info[6] = p.g1; info[7] = p.g2; info[8] = p.g3;
    for (int j = 0; j < 5; ++j) info[9 + j] = p.dl[j];
    info[14] = p.C1Int; info[15] = p.C2Int; info[16] = p.C1MRD; info[17] = p.C2MRD;
  }
  return 0;
}

// IMRPhenomHM container on arbitrary frequencies: mode-major (6, n) hp, hc
// (complex interleaved) and tf, modes (2,2), (2,1), (3,3), (3,2), (4,4), (4,3);
// amp_psi (optional): (6, n, 2) amplitude and phase (h_lm = A exp(-i Psi));
// info (optional, 6 x 4): per mode fRD_lm, Rholm, the amplitude and phase map corners' Mf.
int oracle_phenomhm(const double* th, const double* f, int64_t n, double f_ref, double f_cut_hz, double* hp,
                    double* hc, double* tf, double* amp_psi, double* info) {
  PhenomHM<double> h;
  phenomhm_setup<double>(th, f_ref, h);
  for (int k = 0; k < HM_MODES; ++k) {
    for (int64_t i = 0; i < n; ++i) {
      double amp = 0.0, psi = 0.0, t = 0.0;
      const size_t o = (size_t)k * n + i;
      if (phenomhm_mode<double>(h, k, f[i], f_cut_hz, amp, psi, t)) {
        const double c = std::cos(psi), sn = std::sin(psi);
        hp[2 * o] = h.md[k].P * amp * c;
        hp[2 * o + 1] = -(h.md[k].P * amp * sn);
        hc[2 * o] = h.md[k].C * amp * sn;
        hc[2 * o + 1] = h.md[k].C * amp * c;
      } else {
        hp[2 * o] = hp[2 * o + 1] = hc[2 * o] = hc[2 * o + 1] = 0.0;
      }
      tf[o] = t;
      if (amp_psi) { amp_psi[2 * o] = amp; amp_psi[2 * o + 1] = psi; }
    }
    if (info) {
      info[4 * k] = h.md[k].fRD;
      info[4 * k + 1] = h.md[k].Rholm;
      info[4 * k + 2] = h.md[k].fiA;
      info[4 * k + 3] = h.md[k].frP;
    }
  }
  return 0;
}

// Dense A/E/T (or X/Y/Z) model of one detector for one parameter set.
int oracle_model_tdi(const OraclePlan* pl, int det, int orth, const double* th, double* out) {
  OracleWave<double> wv;
  wave_setup<double>(pl->approximant, th, pl->f_ref, wv);
  double sb = th[7], cb = std::sqrt((1.0 - sb) * (1.0 + sb));
  double P[3][3], X[3][3], k[3];
  polarization<double>(th[6], sb, cb, th[8], P, X, k);
  double fmax = double(pl->k0 + pl->nbins - 1) * pl->f_step + 1.0;
  double fcut = wave_cut_hz(wv, pl->cut_factor, fmax);
  const OracleDet& d = pl->dets[det];
  for (int64_t i = 0; i < pl->nbins; ++i) {
    double f = double(pl->k0 + i) * pl->f_step;
    Cx<double> hp[HM_MODES], hc[HM_MODES], h[3] = {{0, 0}, {0, 0}, {0, 0}};
    double tf[HM_MODES];
    bool live;
    const int nm = wave_eval(wv, f, fcut, hp, hc, tf, &live);
    if (live) {
      Cx<double> L[6];
      response_at_f<double>(d.orbit, f, nm, hp, hc, tf, th[10], P, X, k, L);
      tdi_at_f<double>(f, d.orbit.arm_sec, d.gen20, orth, L, h);
    }
    for (int c = 0; c < 3; ++c) { out[2 * (c * pl->nbins + i)] = h[c].re; out[2 * (c * pl->nbins + i) + 1] = h[c].im; }
  }
  return 0;
}

// Batched lnL (and optionally its exact gradient by forward-mode duals).
int oracle_lnl_batch(const OraclePlan* pl, const double* th, int64_t B, double* lnl, double* grad, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t b = 0; b < B; ++b) {
    const double* t = th + 11 * b;
    if (grad) {
      Dual<11> td[11];
      for (int j = 0; j < 11; ++j) { td[j] = Dual<11>(t[j]); td[j].d[j] = 1.0; }
      Dual<11> r = lnl_one<Dual<11>>(*pl, td);
      lnl[b] = r.v;
      for (int j = 0; j < 11; ++j) grad[11 * b + j] = r.d[j];
    } else {
      lnl[b] = lnl_one<double>(*pl, t);
    }
  }
  return 0;
}

int oracle_fisher_batch(const OraclePlan* pl, const double* th, int64_t B, double* F, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t b = 0; b < B; ++b) fisher_one(*pl, th + 11 * b, F + 121 * b);
  return 0;
}

int oracle_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
