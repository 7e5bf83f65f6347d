// lbm_collide.cuh - per-node arithmetic shared by the fused stream+collide
// kernels: relaxation coefficients, the MRT collision with Guo forcing in
// moment space, and the direct evaluation of the low-wavenumber body force.
#pragma once
#include <cmath>
#include <type_traits>

#include "lbm_internal.cuh"

namespace lbm {
namespace {

template <typename T>
struct Vec2 { T x, y; };

// Relaxation rates of the 15 non-conserved moments in the kernel's own
// precision, folded with the scale factors of the inverse transform.  With
// c_k the factor by which collision.f90:137-157 scales moment k (1/2394,
// 1/252, 1/40 x3, 1/36, 1/72, 1/12, 1/24, 1/4 x3, 1/8 x3) the scaled
// post-collision moment is
//   M_k = c_k [ m_k - s_k (m_k - meq_k) + (1 - s_k/2) mF_k ]
//       = A_k m_k + c_k s_k meq_k + c_k (1 - s_k/2) mF_k,
// and the constant factors inside meq_k and mF_k are folded in as well.
template <typename T>
struct RatesT {
  T A[16];                 // c_k (1 - s_k)
  T B1r, B1t, H1;          // meq1 = -11 rho + 19 t1, mF1 = 38 G3
  T B2r, B2t, H2;          // meq2 = omegepsl rho + omegepslj t1, mF2 = -11 G3
  T B3, H3;                // meq3..5 = -2/3 u, mF3..5 = -2/3 F
  T B6, H6;                // meq6, mF6 = 2 e6
  T B7, H7;                // meq7 = omegxx meq6, mF7 = -e6
  T B8, H8;                // meq8, mF8 = 2 e8
  T B9, H9;                // meq9 = omegxx meq8, mF9 = -e8
  T B10, H10;              // meq10..12 = u_a u_b, mF = F_a u_b + F_b u_a
  // the same factors of the terms linear in the populations as exact
  // fixed-point integers c * 2^sh (FP64 fixed-point collision, collide_fx):
  // [1..15] A_k, [16] B1r, [17] B2r, [18] 1/19
  long long Li[19];
  int Lsh[19];
  // the factors of the velocity and force terms, for the all-integer core
  // (fx_core_int): B1t H1 B2t H2 B3 H3 B6 H6 B7 H7 B8 H8 B9 H9 B10 H10 0.1 0.05
  long long Ni[18];
  int Nsh[18];
  // the same factors at the one scale 2^62 (|c| < 2), so that every product
  // of the integer core shifts by a compile-time amount: [0..18] as Li,
  // [19..36] as Ni
  long long Ci[37];
};

// c as (integer m, shift sh) with c = m * 2^-sh exactly and |m| in
// [2^61, 2^62) (m = 0, sh = 64 for c = 0)
inline void fixed_factor(double c, long long* m, int* sh) {
  if (c == 0.0) { *m = 0; *sh = 64; return; }
  int e = 0;
  std::frexp(c, &e);  // |c| in [2^(e-1), 2^e)
  *sh = 62 - e;
  *m = (long long)std::ldexp(c, *sh);  // exact: 53 significant bits
}

template <typename T>
RatesT<T> rates_t(const Rates& r) {
  RatesT<T> o;
  const double sk[16] = {0.0, r.s1, r.s2, r.s4, r.s4, r.s4, r.s9, r.s10, r.s9, r.s10,
                         r.s13, r.s13, r.s13, r.s16, r.s16, r.s16};
  const double ck[16] = {0.0, 1.0 / 2394.0, 1.0 / 252.0, 1.0 / 40.0, 1.0 / 40.0, 1.0 / 40.0,
                         1.0 / 36.0, 1.0 / 72.0, 1.0 / 12.0, 1.0 / 24.0, 0.25, 0.25, 0.25,
                         0.125, 0.125, 0.125};
  auto Bk = [&](int k) { return ck[k] * sk[k]; };
  auto Hk = [&](int k) { return ck[k] * (1.0 - 0.5 * sk[k]); };
  for (int k = 0; k < 16; ++k) o.A[k] = T(ck[k] * (1.0 - sk[k]));
  o.B1r = T(-11.0 * Bk(1)); o.B1t = T(19.0 * Bk(1)); o.H1 = T(38.0 * Hk(1));
  o.B2r = T(r.omegepsl * Bk(2)); o.B2t = T(r.omegepslj * Bk(2)); o.H2 = T(-11.0 * Hk(2));
  o.B3 = T(-2.0 / 3.0 * Bk(3)); o.H3 = T(-2.0 / 3.0 * Hk(3));
  o.B6 = T(Bk(6)); o.H6 = T(2.0 * Hk(6));
  o.B7 = T(r.omegxx * Bk(7)); o.H7 = T(-Hk(7));
  o.B8 = T(Bk(8)); o.H8 = T(2.0 * Hk(8));
  o.B9 = T(r.omegxx * Bk(9)); o.H9 = T(-Hk(9));
  o.B10 = T(Bk(10)); o.H10 = T(Hk(10));
  for (int k = 0; k < 16; ++k) fixed_factor(ck[k] * (1.0 - sk[k]), &o.Li[k], &o.Lsh[k]);
  fixed_factor(-11.0 * Bk(1), &o.Li[16], &o.Lsh[16]);
  fixed_factor(r.omegepsl * Bk(2), &o.Li[17], &o.Lsh[17]);
  fixed_factor(1.0 / 19.0, &o.Li[18], &o.Lsh[18]);
  const double nf[18] = {19.0 * Bk(1), 38.0 * Hk(1), r.omegepslj * Bk(2), -11.0 * Hk(2),
                         -2.0 / 3.0 * Bk(3), -2.0 / 3.0 * Hk(3), Bk(6), 2.0 * Hk(6),
                         r.omegxx * Bk(7), -Hk(7), Bk(8), 2.0 * Hk(8), r.omegxx * Bk(9), -Hk(9),
                         Bk(10), Hk(10), 0.1, 0.05};
  for (int k = 0; k < 18; ++k) fixed_factor(nf[k], &o.Ni[k], &o.Nsh[k]);
  auto c62 = [](double c) { return (long long)std::llround(std::ldexp(c, 62)); };
  for (int k = 0; k < 16; ++k) o.Ci[k] = c62(ck[k] * (1.0 - sk[k]));
  o.Ci[16] = c62(-11.0 * Bk(1));
  o.Ci[17] = c62(r.omegepsl * Bk(2));
  o.Ci[18] = c62(1.0 / 19.0);
  for (int k = 0; k < 18; ++k) o.Ci[19 + k] = c62(nf[k]);
  return o;
}

// MRT collision with Guo forcing in moment space.  Algebraically the
// collision_MRT of collision.f90:36-203: there f9 = f + Fbar/2 is relaxed in
// moment space, transformed back with rho and u from macrovar, and Fbar/2 is
// added again.  The moments of Fbar have the closed form
//   m1 = 38 u.F, m2 = -11 u.F, m3..5 = -2/3 F, m6 = 2(2 Fx ux - Fy uy - Fz uz),
//   m7 = -m6/2, m8 = 2(Fy uy - Fz uz), m9 = -m8/2, m10 = Fx uy + Fy ux,
//   m11 = Fy uz + Fz uy, m12 = Fx uz + Fz ux, m13..15 = 0,
// with mass 0 and momentum F, so the whole step is one forward transform,
// m'_k = m_k - s_k (m_k - meq_k) + (1 - s_k/2) mF_k, and one inverse
// transform with momentum u + F/2.  This removes the per-direction forcing
// arithmetic, which matters most in FP64 where the GPU's FP64 issue rate
// bounds the kernel.  Results agree with the literal form to rounding.
//   f       in: post-streaming populations; out: post-collision populations
//   fp*     body force of the previous step (macrovar's u = j + Fp/2)
//   f*      body force of this step
template <typename T>
__host__ __device__ __forceinline__ void collide_fast(T (&f)[NPOP], T fpx, T fpy, T fpz, T fx, T fy,
                                             T fz, const RatesT<T>& r) {
  const T a1 = f[1] + f[2], d1 = f[1] - f[2];
  const T a3 = f[3] + f[4], d3 = f[3] - f[4];
  const T a5 = f[5] + f[6], d5 = f[5] - f[6];
  const T s78 = f[7] + f[8], d78 = f[7] - f[8], s910 = f[9] + f[10], d910 = f[9] - f[10];
  const T s1112 = f[11] + f[12], d1112 = f[11] - f[12];
  const T s1314 = f[13] + f[14], d1314 = f[13] - f[14];
  const T s1516 = f[15] + f[16], d1516 = f[15] - f[16];
  const T s1718 = f[17] + f[18], d1718 = f[17] - f[18];
  const T sum1 = a1 + a3 + a5;
  const T Sxy = s78 + s910, Sxz = s1112 + s1314, Syz = s1516 + s1718;
  const T sum2 = Sxy + Sxz + Syz;
  const T D1 = d78 + d910, D2 = d1112 + d1314;
  const T sum3 = D1 + D2;
  const T A = s78 - s910, Bv = d1516 + d1718;
  const T sum4 = A + Bv;
  const T C = s1112 - s1314, Dd = s1516 - s1718;
  const T sum5 = C + Dd;
  const T rho = f[0] + sum1 + sum2;
  // macrovar: u = sum c f + F_prev / 2
  const T ux = d1 + sum3 + T(0.5) * fpx;
  const T uy = d3 + sum4 + T(0.5) * fpy;
  const T uz = d5 + sum5 + T(0.5) * fpz;

  // moments of f (collision.f90:101-118)
  const T sum7 = a3 + a5, sum8 = Sxy + Sxz, sum10 = a3 - a5, sum11 = Sxy - Sxz;
  const T ev1 = T(-30.0) * f[0] + T(-11.0) * sum1 + T(8.0) * sum2;
  const T ev2 = T(12.0) * f[0] + T(-4.0) * sum1 + sum2;
  const T ev3 = T(-4.0) * d1 + sum3;
  const T ev4 = T(-4.0) * d3 + sum4;
  const T ev5 = T(-4.0) * d5 + sum5;
  const T ev6 = T(2.0) * (a1 - Syz) - sum7 + sum8;
  const T ev7 = T(-4.0) * a1 + T(2.0) * (sum7 - Syz) + sum8;
  const T ev8 = sum10 + sum11;
  const T ev9 = T(-2.0) * sum10 + sum11;
  const T ev10 = d78 - d910;
  const T ev11 = d1516 - d1718;
  const T ev12 = d1112 - d1314;
  const T ev13 = D1 - D2;
  const T ev14 = Bv - A;
  const T ev15 = C - Dd;

  // equilibrium (collision.f90:66-81) and forcing moments, shared terms
  const T uxs = ux * ux, uys = uy * uy, uzs = uz * uz;
  const T t1 = uxs + uys + uzs;
  const T eq6 = T(2.0) * uxs - uys - uzs;
  const T eq8 = uys - uzs;
  const T fa = fx * ux, fb = fy * uy, fc = fz * uz;
  const T G3 = fa + fb + fc;
  const T e6 = T(2.0) * fa - fb - fc;
  const T e8 = fb - fc;

  // scaled post-collision moments M_k = tl of collision.f90:138-157
  const T M1 = r.A[1] * ev1 + r.B1r * rho + r.B1t * t1 + r.H1 * G3;
  const T M2 = r.A[2] * ev2 + r.B2r * rho + r.B2t * t1 + r.H2 * G3;
  const T M3 = r.A[3] * ev3 + r.B3 * ux + r.H3 * fx;
  const T M4 = r.A[4] * ev4 + r.B3 * uy + r.H3 * fy;
  const T M5 = r.A[5] * ev5 + r.B3 * uz + r.H3 * fz;
  const T M6 = r.A[6] * ev6 + r.B6 * eq6 + r.H6 * e6;
  const T M7 = r.A[7] * ev7 + r.B7 * eq6 + r.H7 * e6;
  const T M8 = r.A[8] * ev8 + r.B8 * eq8 + r.H8 * e8;
  const T M9 = r.A[9] * ev9 + r.B9 * eq8 + r.H9 * e8;
  const T M10 = r.A[10] * ev10 + uy * (r.B10 * ux + r.H10 * fx) + r.H10 * fy * ux;
  const T M11 = r.A[11] * ev11 + uz * (r.B10 * uy + r.H10 * fy) + r.H10 * fz * uy;
  const T M12 = r.A[12] * ev12 + uz * (r.B10 * ux + r.H10 * fx) + r.H10 * fz * ux;
  const T M13 = r.A[13] * ev13;
  const T M14 = r.A[14] * ev14;
  const T M15 = r.A[15] * ev15;

  // inverse transform (collision.f90:160-200) with momentum u + F/2
  const T tl1 = T(1.0 / 19.0) * rho;
  const T tl6 = T(0.1) * ux + T(0.05) * fx;
  const T tl8 = T(0.1) * uy + T(0.05) * fy;
  const T tl10 = T(0.1) * uz + T(0.05) * fz;

  f[0] = tl1 + T(-30.0) * M1 + T(12.0) * M2;
  const T suma = tl1 + T(-11.0) * M1 + T(-4.0) * M2;
  const T sumb = tl1 + T(8.0) * M1 + M2;
  const T sumc = tl6 - T(4.0) * M3;
  const T sumd = T(2.0) * M6 - T(4.0) * M7;
  const T sume = tl8 - T(4.0) * M4;
  const T q67 = T(2.0) * M7 - M6, r89 = M8 - T(2.0) * M9;
  const T sumf = q67 + r89;
  const T sumg = tl10 - T(4.0) * M5;
  const T sumh = q67 - r89;
  const T p67 = M6 + M7, p89 = M8 + M9;
  const T sumi = p67 + p89;
  const T sumk = p67 - p89;
  const T sump = T(-2.0) * p67;
  const T sum67 = tl6 + M3, sum89 = tl8 + M4, sum1011 = tl10 + M5;
  const T tl16 = M10, tl17 = M11, tl18 = M12, tl19 = M13, tl20 = M14, tl21 = M15;

  const T ad = suma + sumd, af = suma + sumf, ah = suma + sumh;
  f[1] = ad + sumc;
  f[2] = ad - sumc;
  f[3] = af + sume;
  f[4] = af - sume;
  f[5] = ah + sumg;
  f[6] = ah - sumg;
  {  // x-y diagonals 7..10
    const T base = sumb + sumi, p = sum67 + sum89, m = sum67 - sum89;
    const T r1 = tl19 - tl20, r2 = tl19 + tl20;
    f[7] = base + p + tl16 + r1;
    f[8] = base - m - tl16 - r2;
    f[9] = base + m - tl16 + r2;
    f[10] = base - p + tl16 - r1;
  }
  {  // x-z diagonals 11..14
    const T base = sumb + sumk, p = sum67 + sum1011, m = sum67 - sum1011;
    const T r1 = tl21 - tl19, r2 = tl19 + tl21;
    f[11] = base + p + tl18 + r1;
    f[12] = base - m - tl18 + r2;
    f[13] = base + m - tl18 - r2;
    f[14] = base - p + tl18 - r1;
  }
  {  // y-z diagonals 15..18
    const T base = sumb + sump, p = sum89 + sum1011, m = sum89 - sum1011;
    const T r1 = tl20 - tl21, r2 = tl20 + tl21;
    f[15] = base + p + tl17 + r1;
    f[16] = base - m - tl17 - r2;
    f[17] = base + m - tl17 + r2;
    f[18] = base - p + tl17 - r1;
  }
}

// ---------------------------------------------------------------------------
// FP64 collision with error-free integer sums.
//
// GB300 issues FP64 at about 2 lanes per clock per SM and 32-bit integer work
// at 64, so the FP64 kernel is bound by its FP64 instruction count.  Two
// thirds of those instructions are the sums with small integer coefficients
// of the forward and inverse moment transforms.  collide_fx computes those
// sums exactly in 64-bit fixed point (integer adds, no rounding) and keeps
// every product with a non-integer factor (rates, equilibrium, forcing) in
// FP64.  Conversions between FP64 and fixed point are integer bit operations
// (the hardware conversions run at the FP64 rate):
//   inputs and forward sums  v * 2^-58, inputs |f| < 2^-3, sums |.| < 2^5
//   scaled moments, outputs  v * 2^-61, moments |M| < 2^-5, sums |.| < 2^2
// Input rounding is at most 2^-59 and moment rounding 2^-62 in absolute
// terms, the size of the FP64 rounding of the same sums at the populations'
// magnitudes (~1e-2), so results agree with collide_fast to rounding.  A
// node whose inputs or moments leave these ranges (or are not finite), or
// whose populations are all below 2^-12 in magnitude (where the fixed
// point's absolute resolution would cost relative precision), is reported
// by a false return with f untouched; the caller then collides it with
// collide_fast.

constexpr int kFxIn = 58, kFxInMax = -3;    // inputs, forward transform
constexpr int kFxOut = 61, kFxOutMax = -5;  // scaled moments, inverse transform
// a node whose largest |f| is below 2^kFxMinExp keeps FP64's relative
// precision through the FP64 path (fixed point resolves 2^-61 absolute)
constexpr int kFxMinExp = -12;

// x -> round(x * 2^K) (half away from zero); emax collects the largest
// biased exponent seen (the caller tests the range once for all values).
// Values below 2^(-K-1) (zero, subnormals) give 0.
template <int K>
__host__ __device__ __forceinline__ long long fx_from(double x, int& emax) {
  unsigned long long b;
  memcpy(&b, &x, 8);
  const int e = (int)(b >> 52) & 0x7ff;
  emax = emax > e ? emax : e;
  // magnitude with the hidden bit at bit 63: |x| = m * 2^(e - 1086)
  const unsigned long long m = (b << 11) | 0x8000000000000000ULL;
  // |x| * 2^K = m * 2^-(1086 - K - e): shift by one less, add the half, shift
  const int r1 = 1085 - K - e;  // >= 0 inside the range
  const unsigned long long v = ((unsigned)r1 >= 64u ? 0ULL : (m >> r1) + 1) >> 1;
  const long long sg = (long long)b >> 63;  // 0 or -1
  return ((long long)v ^ sg) - sg;
}

// v * 2^-K as a double, rounded to nearest (ties away from zero)
template <int K>
__host__ __device__ __forceinline__ double fx_to(long long v) {
  const long long sg = v >> 63;
  unsigned long long a = (unsigned long long)((v ^ sg) - sg);
#ifdef __CUDA_ARCH__
  const int lz = __clzll((long long)a);
#else
  const int lz = a ? __builtin_clzll(a) : 64;
#endif
  a = lz >= 64 ? 0ULL : a << lz;  // leading one at bit 63
  // 53 bits with the hidden one, rounded on bit 10; a carry to 2^53 adds one
  // to the exponent field through the sum below
  const unsigned long long mant = (a >> 11) + ((a >> 10) & 1ULL);
  const unsigned long long E = (unsigned long long)(1086 - K - lz);  // biased exponent
  const unsigned long long bits =
      ((unsigned long long)sg << 63) | (((E - 1) << 52) + mant);
  double d;
  memcpy(&d, &bits, 8);
  return a ? d : 0.0;
}


// round(v * m * 2^-sh_total) with v a fixed-point value (scale 2^-kFxIn),
// (m, sh) a fixed_factor, the result at scale 2^-kFxOut: one exact 128-bit
// product and one rounding
__host__ __device__ __forceinline__ long long fx_mul(long long v, long long m, int sh) {
  const int s = sh + kFxIn - kFxOut;  // >= 1: |c| < 2^58
  const __int128 p = (__int128)v * (__int128)m + ((__int128)1 << (s - 1));
  return (long long)(p >> s);
}

// |x| < 2^(kFxOutMax) at scale 2^-kFxOut
__host__ __device__ __forceinline__ unsigned fx_out_of_range(long long x) {
  // |x| >= 2^(kFxOut + kFxOutMax) = 2^56, on the high word: the bound's low
  // word is zero, so x + 2^56 >= 2^57 is (hi + 2^24) >= 2^25 in 32 bits
  constexpr unsigned hlim = 1u << (kFxOut + kFxOutMax - 32);
  return ((unsigned)((unsigned long long)x >> 32) + hlim) & ~(2 * hlim - 1);
}

// The collision of collide_fast with the integer-coefficient sums of both
// transforms exact in fixed point, and the terms linear in the populations
// (A_k m_k, the density terms of meq1, meq2 and rho / 19) as exact integer
// products rounded once (RatesT::Li); only the terms with velocities and
// forces stay FP64.  Returns false, leaving f as it was, when a value is
// out of the fixed-point ranges.
//
// fx_core is the part between the conversions: g the populations at scale
// 2^-kFxIn (|g| < 2^(kFxIn + kFxInMax)), h the post-collision populations at
// 2^-kFxOut; false when a moment leaves its range.  The previous step's body
// force fp (the velocity's F/2) is FP64, or (FP = long long) fixed point at
// 2^-kFxF, added to the momentum sums exactly.
constexpr int kFxF = 70;  // body forces in fixed point: |F| < 2^-7 at 2^-70
template <typename FP>
__host__ __device__ __forceinline__ bool fx_core(const long long (&g)[NPOP], FP fpx, FP fpy,
                                                 FP fpz, double fx, double fy, double fz,
                                                 const RatesT<double>& r, long long (&h)[NPOP]) {
  typedef long long I;
  int emax = 0;
  // forward transform, exact (collision.f90:101-118; grouping as collide_fast)
  const I a1 = g[1] + g[2], d1 = g[1] - g[2];
  const I a3 = g[3] + g[4], d3 = g[3] - g[4];
  const I a5 = g[5] + g[6], d5 = g[5] - g[6];
  const I s78 = g[7] + g[8], d78 = g[7] - g[8], s910 = g[9] + g[10], d910 = g[9] - g[10];
  const I s1112 = g[11] + g[12], d1112 = g[11] - g[12];
  const I s1314 = g[13] + g[14], d1314 = g[13] - g[14];
  const I s1516 = g[15] + g[16], d1516 = g[15] - g[16];
  const I s1718 = g[17] + g[18], d1718 = g[17] - g[18];
  const I sum1 = a1 + a3 + a5;
  const I Sxy = s78 + s910, Sxz = s1112 + s1314, Syz = s1516 + s1718;
  const I sum2 = Sxy + Sxz + Syz;
  const I D1 = d78 + d910, D2 = d1112 + d1314;
  const I sum3 = D1 + D2;
  const I A = s78 - s910, Bv = d1516 + d1718;
  const I sum4 = A + Bv;
  const I C = s1112 - s1314, Dd = s1516 - s1718;
  const I sum5 = C + Dd;
  const I sum7 = a3 + a5, sum8 = Sxy + Sxz, sum10 = a3 - a5, sum11 = Sxy - Sxz;
  const I rho = g[0] + sum1 + sum2;
  const I ev1 = -30 * g[0] - 11 * sum1 + 8 * sum2;
  const I ev2 = 12 * g[0] - 4 * sum1 + sum2;
  const I ev3 = -4 * d1 + sum3;
  const I ev4 = -4 * d3 + sum4;
  const I ev5 = -4 * d5 + sum5;
  const I ev6 = 2 * (a1 - Syz) - sum7 + sum8;
  const I ev7 = -4 * a1 + 2 * (sum7 - Syz) + sum8;
  const I ev8 = sum10 + sum11;
  const I ev9 = -2 * sum10 + sum11;
  // macrovar: u = sum c f + F_prev / 2
  double ux, uy, uz;
  if constexpr (std::is_integral<FP>::value) {
    // F/2 from 2^-kFxF to 2^-kFxIn, rounded
    constexpr int sh = kFxF - kFxIn + 1;
    auto half = [](long long v) { return (v + (1LL << (sh - 1))) >> sh; };
    ux = fx_to<kFxIn>(d1 + sum3 + half(fpx));
    uy = fx_to<kFxIn>(d3 + sum4 + half(fpy));
    uz = fx_to<kFxIn>(d5 + sum5 + half(fpz));
  } else {
    ux = fx_to<kFxIn>(d1 + sum3) + 0.5 * fpx;
    uy = fx_to<kFxIn>(d3 + sum4) + 0.5 * fpy;
    uz = fx_to<kFxIn>(d5 + sum5) + 0.5 * fpz;
  }

  // equilibrium and forcing moments, FP64 (collision.f90:66-81)
  const double uxs = ux * ux, uys = uy * uy, uzs = uz * uz;
  const double t1 = uxs + uys + uzs;
  const double eq6 = 2.0 * uxs - uys - uzs;
  const double eq8 = uys - uzs;
  const double fa = fx * ux, fb = fy * uy, fc = fz * uz;
  const double G3 = fa + fb + fc;
  const double e6 = 2.0 * fa - fb - fc;
  const double e8 = fb - fc;

  // scaled post-collision moments (collision.f90:138-157): the linear part
  // as integer products, the rest converted from FP64
  auto L = [&](int k, I v) { return fx_mul(v, r.Li[k], r.Lsh[k]); };
  auto F = [&](double x) { return fx_from<kFxOut>(x, emax); };
  I M[16];
  M[1] = L(1, ev1) + L(16, rho) + F(r.B1t * t1 + r.H1 * G3);
  M[2] = L(2, ev2) + L(17, rho) + F(r.B2t * t1 + r.H2 * G3);
  M[3] = L(3, ev3) + F(r.B3 * ux + r.H3 * fx);
  M[4] = L(4, ev4) + F(r.B3 * uy + r.H3 * fy);
  M[5] = L(5, ev5) + F(r.B3 * uz + r.H3 * fz);
  M[6] = L(6, ev6) + F(r.B6 * eq6 + r.H6 * e6);
  M[7] = L(7, ev7) + F(r.B7 * eq6 + r.H7 * e6);
  M[8] = L(8, ev8) + F(r.B8 * eq8 + r.H8 * e8);
  M[9] = L(9, ev9) + F(r.B9 * eq8 + r.H9 * e8);
  M[10] = L(10, d78 - d910) + F(uy * (r.B10 * ux + r.H10 * fx) + r.H10 * fy * ux);
  M[11] = L(11, d1516 - d1718) + F(uz * (r.B10 * uy + r.H10 * fy) + r.H10 * fz * uy);
  M[12] = L(12, d1112 - d1314) + F(uz * (r.B10 * ux + r.H10 * fx) + r.H10 * fz * ux);
  M[13] = L(13, D1 - D2);
  M[14] = L(14, Bv - A);
  M[15] = L(15, C - Dd);
  const I tl1 = L(18, rho);
  const I tl6 = F(0.1 * ux + 0.05 * fx);
  const I tl8 = F(0.1 * uy + 0.05 * fy);
  const I tl10 = F(0.1 * uz + 0.05 * fz);
  unsigned out = emax >= 1023 - 1;  // FP64 parts below 1/2
#pragma unroll
  for (int k = 1; k < 16; ++k) out |= fx_out_of_range(M[k]);
  out |= fx_out_of_range(tl1) | fx_out_of_range(tl6) | fx_out_of_range(tl8) |
         fx_out_of_range(tl10);
  if (out) return false;

  // inverse transform, exact (collision.f90:160-200)
  h[0] = tl1 - 30 * M[1] + 12 * M[2];
  const I suma = tl1 - 11 * M[1] - 4 * M[2];
  const I sumb = tl1 + 8 * M[1] + M[2];
  const I sumc = tl6 - 4 * M[3];
  const I sumd = 2 * M[6] - 4 * M[7];
  const I sume = tl8 - 4 * M[4];
  const I q67 = 2 * M[7] - M[6], r89 = M[8] - 2 * M[9];
  const I sumf = q67 + r89;
  const I sumg = tl10 - 4 * M[5];
  const I sumh = q67 - r89;
  const I p67 = M[6] + M[7], p89 = M[8] + M[9];
  const I sumi = p67 + p89;
  const I sumk = p67 - p89;
  const I sump = -2 * p67;
  const I sum67 = tl6 + M[3], sum89 = tl8 + M[4], sum1011 = tl10 + M[5];
  const I ad = suma + sumd, af = suma + sumf, ah = suma + sumh;
  h[1] = ad + sumc;
  h[2] = ad - sumc;
  h[3] = af + sume;
  h[4] = af - sume;
  h[5] = ah + sumg;
  h[6] = ah - sumg;
  {  // x-y diagonals 7..10
    const I base = sumb + sumi, p = sum67 + sum89, m = sum67 - sum89;
    const I bp = base + M[10], bm = base - M[10];
    const I P = p + (M[13] - M[14]), Q = m + (M[13] + M[14]);
    h[7] = bp + P;
    h[10] = bp - P;
    h[8] = bm - Q;
    h[9] = bm + Q;
  }
  {  // x-z diagonals 11..14
    const I base = sumb + sumk, p = sum67 + sum1011, m = sum67 - sum1011;
    const I bp = base + M[12], bm = base - M[12];
    const I P = p + (M[15] - M[13]), Q = m - (M[13] + M[15]);
    h[11] = bp + P;
    h[14] = bp - P;
    h[12] = bm - Q;
    h[13] = bm + Q;
  }
  {  // y-z diagonals 15..18
    const I base = sumb + sump, p = sum89 + sum1011, m = sum89 - sum1011;
    const I bp = base + M[11], bm = base - M[11];
    const I P = p + (M[14] - M[15]), Q = m + (M[14] + M[15]);
    h[15] = bp + P;
    h[18] = bp - P;
    h[16] = bm - Q;
    h[17] = bm + Q;
  }
  return true;
}

// round(a * b * 2^-s), s >= 1: one exact 128-bit product, one rounding.
// (An explicit carry chain, mad.lo.cc / madc.hi with the rounding constant
// as the addend, measured 8 % slower for the whole FP64 step than this.)
__host__ __device__ __forceinline__ long long mul_round(long long a, long long b, int s) {
  const __int128 p = (__int128)a * (__int128)b + ((__int128)1 << (s - 1));
  return (long long)(p >> s);
}

// fx_core with the velocity and force terms as integer products too, so the
// collision issues no FP64 instruction: the velocity u (scale 2^-kFxIn) and
// this step's body force F (2^-kFxF) enter as integers; the products
// u_a u_b are rounded once to 2^-64 and F_a u_b to 2^-kFxF; each term of a
// moment is one exact 128-bit product of such a value and a fixed-point
// factor (RatesT::Ni), rounded once to 2^-kFxOut.  Ranges, so that nothing
// overflows: |u| < 2^-2 and |F| < 2^-9 (a node beyond them is declined, as
// is one whose moments leave their ranges).  The roundings (2^-62 per term)
// are those of fx_core's conversions from FP64.
constexpr int kFxUU = 64;  // u_a u_b
//
// bias is added to every output (through tl1, which each of them holds once):
// the caller's rounding constant costs one add instead of nineteen.
__host__ __device__ __forceinline__ bool fx_core_int(const long long (&g)[NPOP], long long fpx,
                                                     long long fpy, long long fpz, long long Fx,
                                                     long long Fy, long long Fz,
                                                     const RatesT<double>& r,
                                                     long long (&h)[NPOP], long long bias = 0) {
  typedef long long I;
  const I a1 = g[1] + g[2], d1 = g[1] - g[2];
  const I a3 = g[3] + g[4], d3 = g[3] - g[4];
  const I a5 = g[5] + g[6], d5 = g[5] - g[6];
  const I s78 = g[7] + g[8], d78 = g[7] - g[8], s910 = g[9] + g[10], d910 = g[9] - g[10];
  const I s1112 = g[11] + g[12], d1112 = g[11] - g[12];
  const I s1314 = g[13] + g[14], d1314 = g[13] - g[14];
  const I s1516 = g[15] + g[16], d1516 = g[15] - g[16];
  const I s1718 = g[17] + g[18], d1718 = g[17] - g[18];
  const I sum1 = a1 + a3 + a5;
  const I Sxy = s78 + s910, Sxz = s1112 + s1314, Syz = s1516 + s1718;
  const I sum2 = Sxy + Sxz + Syz;
  const I D1 = d78 + d910, D2 = d1112 + d1314;
  const I sum3 = D1 + D2;
  const I A = s78 - s910, Bv = d1516 + d1718;
  const I sum4 = A + Bv;
  const I C = s1112 - s1314, Dd = s1516 - s1718;
  const I sum5 = C + Dd;
  const I sum7 = a3 + a5, sum8 = Sxy + Sxz, sum10 = a3 - a5, sum11 = Sxy - Sxz;
  const I rho = g[0] + sum1 + sum2;
  const I ev1 = -30 * g[0] - 11 * sum1 + 8 * sum2;
  const I ev2 = 12 * g[0] - 4 * sum1 + sum2;
  const I ev3 = -4 * d1 + sum3;
  const I ev4 = -4 * d3 + sum4;
  const I ev5 = -4 * d5 + sum5;
  const I ev6 = 2 * (a1 - Syz) - sum7 + sum8;
  const I ev7 = -4 * a1 + 2 * (sum7 - Syz) + sum8;
  const I ev8 = sum10 + sum11;
  const I ev9 = -2 * sum10 + sum11;
  // macrovar: u = sum c f + F_prev / 2, exact at 2^-kFxIn
  constexpr int sh = kFxF - kFxIn + 1;
  auto half = [](long long v) { return (v + (1LL << (sh - 1))) >> sh; };
  const I ux = d1 + sum3 + half(fpx);
  const I uy = d3 + sum4 + half(fpy);
  const I uz = d5 + sum5 + half(fpz);
  {
    // |u| < 2^-2 and |F| < 2^-9, on the high words (the bounds' low words are
    // zero, as for the input test of collide_fx_fixed_int)
    constexpr unsigned ulim = 1u << (kFxIn - 2 - 32);
    constexpr unsigned flim = 1u << (kFxF - 9 - 32);
    auto hw = [](long long v) { return (unsigned)((unsigned long long)v >> 32); };
    const unsigned bad = ((hw(ux) + ulim) | (hw(uy) + ulim) | (hw(uz) + ulim)) & ~(2 * ulim - 1);
    const unsigned badf = ((hw(Fx) + flim) | (hw(Fy) + flim) | (hw(Fz) + flim)) & ~(2 * flim - 1);
    if (bad | badf) return false;
  }
  // products (collision.f90:66-81): u_a u_b at 2^-64, F_a u_b at 2^-kFxF
  constexpr int suu = 2 * kFxIn - kFxUU, sfu = kFxIn;
  const I qxx = mul_round(ux, ux, suu), qyy = mul_round(uy, uy, suu), qzz = mul_round(uz, uz, suu);
  const I qxy = mul_round(ux, uy, suu), qyz = mul_round(uy, uz, suu), qxz = mul_round(ux, uz, suu);
  const I pa = mul_round(Fx, ux, sfu), pb = mul_round(Fy, uy, sfu), pc = mul_round(Fz, uz, sfu);
  const I t1 = qxx + qyy + qzz;
  const I eq6 = 2 * qxx - qyy - qzz, eq8 = qyy - qzz;
  const I G3 = pa + pb + pc, e6 = 2 * pa - pb - pc, e8 = pb - pc;
  const I m10 = mul_round(Fx, uy, sfu) + mul_round(Fy, ux, sfu);
  const I m11 = mul_round(Fy, uz, sfu) + mul_round(Fz, uy, sfu);
  const I m12 = mul_round(Fx, uz, sfu) + mul_round(Fz, ux, sfu);
  // factor k (at 2^-62) times a value at scale 2^-sv, at 2^-kFxOut: the
  // shifts are compile-time constants
  auto N = [&](int k, I v, int sv) { return mul_round(v, r.Ci[19 + k], 62 + sv - kFxOut); };
  auto L = [&](int k, I v) { return mul_round(v, r.Ci[k], 62 + kFxIn - kFxOut); };
  I M[16];
  M[1] = L(1, ev1) + L(16, rho) + N(0, t1, kFxUU) + N(1, G3, kFxF);
  M[2] = L(2, ev2) + L(17, rho) + N(2, t1, kFxUU) + N(3, G3, kFxF);
  M[3] = L(3, ev3) + N(4, ux, kFxIn) + N(5, Fx, kFxF);
  M[4] = L(4, ev4) + N(4, uy, kFxIn) + N(5, Fy, kFxF);
  M[5] = L(5, ev5) + N(4, uz, kFxIn) + N(5, Fz, kFxF);
  M[6] = L(6, ev6) + N(6, eq6, kFxUU) + N(7, e6, kFxF);
  M[7] = L(7, ev7) + N(8, eq6, kFxUU) + N(9, e6, kFxF);
  M[8] = L(8, ev8) + N(10, eq8, kFxUU) + N(11, e8, kFxF);
  M[9] = L(9, ev9) + N(12, eq8, kFxUU) + N(13, e8, kFxF);
  M[10] = L(10, d78 - d910) + N(14, qxy, kFxUU) + N(15, m10, kFxF);
  M[11] = L(11, d1516 - d1718) + N(14, qyz, kFxUU) + N(15, m11, kFxF);
  M[12] = L(12, d1112 - d1314) + N(14, qxz, kFxUU) + N(15, m12, kFxF);
  M[13] = L(13, D1 - D2);
  M[14] = L(14, Bv - A);
  M[15] = L(15, C - Dd);
  const I tl1 = L(18, rho);
  const I tl6 = N(16, ux, kFxIn) + N(17, Fx, kFxF);
  const I tl8 = N(16, uy, kFxIn) + N(17, Fy, kFxF);
  const I tl10 = N(16, uz, kFxIn) + N(17, Fz, kFxF);
  unsigned out = 0;
#pragma unroll
  for (int k = 1; k < 16; ++k) out |= fx_out_of_range(M[k]);
  out |= fx_out_of_range(tl1) | fx_out_of_range(tl6) | fx_out_of_range(tl8) |
         fx_out_of_range(tl10);
  if (out) return false;

  // inverse transform, exact (collision.f90:160-200)
  const I tlb = tl1 + bias;
  h[0] = tlb - 30 * M[1] + 12 * M[2];
  const I suma = tlb - 11 * M[1] - 4 * M[2];
  const I sumb = tlb + 8 * M[1] + M[2];
  const I sumc = tl6 - 4 * M[3];
  const I sumd = 2 * M[6] - 4 * M[7];
  const I sume = tl8 - 4 * M[4];
  const I q67 = 2 * M[7] - M[6], r89 = M[8] - 2 * M[9];
  const I sumf = q67 + r89;
  const I sumg = tl10 - 4 * M[5];
  const I sumh = q67 - r89;
  const I p67 = M[6] + M[7], p89 = M[8] + M[9];
  const I sumi = p67 + p89;
  const I sumk = p67 - p89;
  const I sump = -2 * p67;
  const I sum67 = tl6 + M[3], sum89 = tl8 + M[4], sum1011 = tl10 + M[5];
  const I ad = suma + sumd, af = suma + sumf, ah = suma + sumh;
  h[1] = ad + sumc;
  h[2] = ad - sumc;
  h[3] = af + sume;
  h[4] = af - sume;
  h[5] = ah + sumg;
  h[6] = ah - sumg;
  {
    const I base = sumb + sumi, p = sum67 + sum89, m = sum67 - sum89;
    const I bp = base + M[10], bm = base - M[10];
    const I P = p + (M[13] - M[14]), Q = m + (M[13] + M[14]);
    h[7] = bp + P;
    h[10] = bp - P;
    h[8] = bm - Q;
    h[9] = bm + Q;
  }
  {
    const I base = sumb + sumk, p = sum67 + sum1011, m = sum67 - sum1011;
    const I bp = base + M[12], bm = base - M[12];
    const I P = p + (M[15] - M[13]), Q = m - (M[13] + M[15]);
    h[11] = bp + P;
    h[14] = bp - P;
    h[12] = bm - Q;
    h[13] = bm + Q;
  }
  {
    const I base = sumb + sump, p = sum89 + sum1011, m = sum89 - sum1011;
    const I bp = base + M[11], bm = base - M[11];
    const I P = p + (M[14] - M[15]), Q = m + (M[14] + M[15]);
    h[15] = bp + P;
    h[18] = bp - P;
    h[16] = bm - Q;
    h[17] = bm + Q;
  }
  return true;
}

__host__ __device__ __forceinline__ bool collide_fx(double (&f)[NPOP], double fpx, double fpy,
                                                    double fpz, double fx, double fy, double fz,
                                                    const RatesT<double>& r) {
  int emax = 0;
  long long g[NPOP], h[NPOP];
#pragma unroll
  for (int q = 0; q < NPOP; ++q) g[q] = fx_from<kFxIn>(f[q], emax);
  if (emax >= 1023 + kFxInMax || emax < 1023 + kFxMinExp) return false;
  if (!fx_core<double>(g, fpx, fpy, fpz, fx, fy, fz, r, h)) return false;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) f[q] = fx_to<kFxOut>(h[q]);
  return true;
}

// Populations stored as 64-bit fixed point at scale 2^-kFxIn (the FP64 plain
// path between fused steps): |f| < 2^(63 - kFxIn) = 32 is representable, the
// absolute resolution is 2^-58 = 3.5e-18 (FP64's own rounding of populations
// of 0.01 to 0.1 is 1.7e-18 to 1.4e-17).
__host__ __device__ __forceinline__ double pop_from_fixed(long long v) { return fx_to<kFxIn>(v); }
// false when v is not finite or |v| >= 32
__host__ __device__ __forceinline__ bool pop_to_fixed(double v, long long& out) {
  int e = 0;
  out = fx_from<kFxIn>(v, e);
  return e < 1023 + (63 - kFxIn);
}

// collide_fx on populations already in the stored fixed point: no
// conversions in or out (the outputs are rounded from 2^-kFxOut to 2^-kFxIn).
// False, with g as it was, when an input is outside |f| < 2^kFxInMax or a
// moment leaves its range.
template <typename FP>
__host__ __device__ __forceinline__ bool collide_fx_fixed(long long (&g)[NPOP], FP fpx, FP fpy,
                                                          FP fpz, double fx, double fy, double fz,
                                                          const RatesT<double>& r) {
  constexpr unsigned long long lim = 1ULL << (kFxIn + kFxInMax);
  unsigned long long out = 0;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) out |= ((unsigned long long)g[q] + lim) & ~(2 * lim - 1);
  if (out) return false;
  long long h[NPOP];
  if (!fx_core<FP>(g, fpx, fpy, fpz, fx, fy, fz, r, h)) return false;
  constexpr int sh = kFxOut - kFxIn;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) g[q] = (h[q] + (1LL << (sh - 1))) >> sh;
  return true;
}

// collide_fx_fixed with the all-integer core (fx_core_int): the forces of
// this step (Fx, Fy, Fz) at 2^-kFxF.
__host__ __device__ __forceinline__ bool collide_fx_fixed_int(long long (&g)[NPOP], long long fpx,
                                                              long long fpy, long long fpz,
                                                              long long Fx, long long Fy,
                                                              long long Fz,
                                                              const RatesT<double>& r) {
  // |g| < 2^(kFxIn + kFxInMax) = 2^55, tested on the high words: the bound's
  // low word is zero, so g + 2^55 < 2^56 is (hi + 2^23) < 2^24 in 32 bits
  constexpr unsigned hlim = 1u << (kFxIn + kFxInMax - 32);
  unsigned out = 0;
#pragma unroll
  for (int q = 0; q < NPOP; ++q)
    out |= ((unsigned)((unsigned long long)g[q] >> 32) + hlim) & ~(2 * hlim - 1);
  if (out) return false;
  long long h[NPOP];
  constexpr int sh = kFxOut - kFxIn;
  if (!fx_core_int(g, fpx, fpy, fpz, Fx, Fy, Fz, r, h, 1LL << (sh - 1))) return false;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) g[q] = h[q] >> sh;
  return true;
}

// Body force of two fields (previous and current step) at one node, sharing
// the per-x twiddles; see ForceView.
template <typename T>
__device__ __forceinline__ void body_force2(const ForceView<T>& fa, const ForceView<T>& fb,
                                            int x, int row, T (&oa)[3], T (&ob)[3]) {
  T c1 = T(0), s1 = T(0), c2 = T(0), s2 = T(0);
  if (fa.mode == FM_TABLE || fb.mode == FM_TABLE) {
    c1 = fa.xtw[4 * x]; s1 = fa.xtw[4 * x + 1]; c2 = fa.xtw[4 * x + 2]; s2 = fa.xtw[4 * x + 3];
  }
  const ForceView<T>* fv[2] = {&fa, &fb};
  T* out[2] = {oa, ob};
#pragma unroll
  for (int w = 0; w < 2; ++w) {
    const ForceView<T>& v = *fv[w];
    if (v.mode == FM_TABLE) {
      const T* k = v.rowtab + (long long)row * kRowCoef;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        out[w][c] = k[5 * c] + k[5 * c + 1] * c1 + k[5 * c + 2] * s1 + k[5 * c + 3] * c2 +
                    k[5 * c + 4] * s2;
    } else if (v.mode == FM_CONST) {
      out[w][0] = v.cfx; out[w][1] = v.cfy; out[w][2] = v.cfz;
    } else {
      out[w][0] = T(0); out[w][1] = T(0); out[w][2] = T(0);
    }
  }
}

}  // namespace
}  // namespace lbm
