// lbm_fluid.cu - fluid kernels of the GB300 lattice Boltzmann engine.
//
// The hot kernel is k_fused: one pass over the box that, per node,
//   1. loads the 19 post-streaming populations (coalesced, x fastest),
//   2. forms rho and u exactly as macrovar does (B/collision.f90:249-271),
//      with the previous step's body force,
//   3. evaluates the current step's body force at the node directly from
//      the low-wavenumber forcing modes (replacing the three inverse FFTs of
//      FORCING, B/gaussian.f90:595-601),
//   4. applies the MRT collision with Guo-type forcing of collision_MRT
//      (B/collision.f90:31-208) at fluid nodes,
//   5. pushes every population to its neighbour (the cshift streaming of
//      B/streaming.f90:13-166), bouncing it back at x walls in the channel
//      (C/streaming.f90:175-187).
// It reads and writes each population once: 2*19*sizeof(T) bytes per node
// plus a 4-byte flag.  In FP64 the MRT arithmetic, not HBM, bounds it on
// GB300, whose FP64 rate is a small fraction of its FP32 rate.
#include "lbm_internal.cuh"
#include "lbm_collide.cuh"

namespace lbm {

namespace {


// MRT collision of one fluid node, B/collision.f90:36-203.  f holds the
// node's 19 populations on entry and the post-collision populations on
// exit.  rho9/ux9.. are the macroscopic values of macrovar, fx9.. the body
// force of the current step.  The arithmetic follows the reference term by
// term (the compiler may fuse multiply-adds).
template <typename T>
__device__ __forceinline__ void collide_mrt(T (&f)[NPOP], T rho9, T ux9, T uy9, T uz9,
                                            T fx9, T fy9, T fz9, const Rates& r) {
  const T ww1 = T(1.0 / 18.0), ww2 = T(1.0 / 36.0);
  const T coef1 = T(-2.0 / 3.0), coef2 = T(-11.0), coef3 = T(8.0), coef4 = T(-4.0), coef5 = T(2.0);
  const T coef3i = T(1.0 / 8.0), coef4i = T(1.0 / -4.0);
  const T val1i = T(1.0 / 19.0), val2i = T(1.0 / 2394.0), val3i = T(1.0 / 252.0);
  const T val4i = T(1.0 / 10.0), val5i = T(1.0 / 40.0), val6i = T(1.0 / 36.0);
  const T val7i = T(1.0 / 72.0), val8i = T(1.0 / 12.0), val9i = T(1.0 / 24.0), val8 = T(12.0);
  const T s1 = T(r.s1), s2 = T(r.s2), s4 = T(r.s4), s9 = T(r.s9), s10 = T(r.s10);
  const T s13 = T(r.s13), s16 = T(r.s16);

  T ux9s = ux9 * ux9, uy9s = uy9 * uy9, uz9s = uz9 * uz9;
  T G3 = ux9 * fx9 + uy9 * fy9 + uz9 * fz9;
  T Fbar[NPOP];
  Fbar[0] = -G3;
#pragma unroll
  for (int ip = 1; ip < NPOP; ++ip) {
    T G1 = T(cix(ip)) * fx9 + T(ciy(ip)) * fy9 + T(ciz(ip)) * fz9;
    T G2 = T(cix(ip)) * ux9 + T(ciy(ip)) * uy9 + T(ciz(ip)) * uz9;
    T w = ip <= 6 ? ww1 : ww2;
    Fbar[ip] = w * (T(3.) * G1 + T(9.) * G1 * G2 - T(3.) * G3);
  }
  T f9[NPOP];
#pragma unroll
  for (int ip = 0; ip < NPOP; ++ip) f9[ip] = f[ip] + Fbar[ip] * T(0.5);

  T t1 = ux9s + uy9s + uz9s;
  T eqm1 = T(-11.0) * rho9 + T(19.0) * t1;
  T eqm2 = T(r.omegepsl) * rho9 + T(r.omegepslj) * t1;
  T eqm3 = coef1 * ux9, eqm4 = coef1 * uy9, eqm5 = coef1 * uz9;
  T eqm6 = T(2.0) * ux9s - uy9s - uz9s;
  T eqm7 = T(r.omegxx) * eqm6;
  T eqm8 = uy9s - uz9s;
  T eqm9 = T(r.omegxx) * eqm8;
  T eqm10 = ux9 * uy9, eqm11 = uy9 * uz9, eqm12 = ux9 * uz9;

  T sum1 = f9[1] + f9[2] + f9[3] + f9[4] + f9[5] + f9[6];
  T sum2 = f9[7] + f9[8] + f9[9] + f9[10] + f9[11] + f9[12] + f9[13] + f9[14] + f9[15] +
           f9[16] + f9[17] + f9[18];
  T sum3 = f9[7] - f9[8] + f9[9] - f9[10] + f9[11] - f9[12] + f9[13] - f9[14];
  T sum4 = f9[7] + f9[8] - f9[9] - f9[10] + f9[15] - f9[16] + f9[17] - f9[18];
  T sum5 = f9[11] + f9[12] - f9[13] - f9[14] + f9[15] + f9[16] - f9[17] - f9[18];
  T sum6 = f9[1] + f9[2];
  T sum7 = f9[3] + f9[4] + f9[5] + f9[6];
  T sum8 = f9[7] + f9[8] + f9[9] + f9[10] + f9[11] + f9[12] + f9[13] + f9[14];
  T sum9 = f9[15] + f9[16] + f9[17] + f9[18];
  T sum10 = f9[3] + f9[4] - f9[5] - f9[6];
  T sum11 = f9[7] + f9[8] + f9[9] + f9[10] - f9[11] - f9[12] - f9[13] - f9[14];

  T evlm1 = T(-30.0) * f9[0] + coef2 * sum1 + coef3 * sum2;
  T evlm2 = T(12.0) * f9[0] + coef4 * sum1 + sum2;
  T evlm3 = coef4 * (f9[1] - f9[2]) + sum3;
  T evlm4 = coef4 * (f9[3] - f9[4]) + sum4;
  T evlm5 = coef4 * (f9[5] - f9[6]) + sum5;
  T evlm6 = coef5 * sum6 - sum7 + sum8 - coef5 * sum9;
  T evlm7 = coef4 * sum6 + coef5 * sum7 + sum8 - coef5 * sum9;
  T evlm8 = sum10 + sum11;
  T evlm9 = -coef5 * sum10 + sum11;
  T evlm10 = f9[7] - f9[8] - f9[9] + f9[10];
  T evlm11 = f9[15] - f9[16] - f9[17] + f9[18];
  T evlm12 = f9[11] - f9[12] - f9[13] + f9[14];
  T evlm13 = f9[7] - f9[8] + f9[9] - f9[10] - f9[11] + f9[12] - f9[13] + f9[14];
  T evlm14 = -f9[7] - f9[8] + f9[9] + f9[10] + f9[15] - f9[16] + f9[17] - f9[18];
  T evlm15 = f9[11] + f9[12] - f9[13] - f9[14] - f9[15] - f9[16] + f9[17] + f9[18];

  T eqmc1 = evlm1 - s1 * (evlm1 - eqm1);
  T eqmc2 = evlm2 - s2 * (evlm2 - eqm2);
  T eqmc3 = evlm3 - s4 * (evlm3 - eqm3);
  T eqmc4 = evlm4 - s4 * (evlm4 - eqm4);
  T eqmc5 = evlm5 - s4 * (evlm5 - eqm5);
  T eqmc6 = evlm6 - s9 * (evlm6 - eqm6);
  T eqmc7 = evlm7 - s10 * (evlm7 - eqm7);
  T eqmc8 = evlm8 - s9 * (evlm8 - eqm8);
  T eqmc9 = evlm9 - s10 * (evlm9 - eqm9);
  T eqmc10 = evlm10 - s13 * (evlm10 - eqm10);
  T eqmc11 = evlm11 - s13 * (evlm11 - eqm11);
  T eqmc12 = evlm12 - s13 * (evlm12 - eqm12);
  T eqmc13 = evlm13 - s16 * evlm13;
  T eqmc14 = evlm14 - s16 * evlm14;
  T eqmc15 = evlm15 - s16 * evlm15;

  T tl1 = val1i * rho9;
  T tl2 = coef2 * val2i * eqmc1;
  T tl3 = coef3 * val2i * eqmc1;
  T tl4 = coef4 * val3i * eqmc2;
  T tl5 = val3i * eqmc2;
  T tl6 = val4i * ux9;
  T tl7 = val5i * eqmc3;
  T tl8 = val4i * uy9;
  T tl9 = val5i * eqmc4;
  T tl10 = val4i * uz9;
  T tl11 = val5i * eqmc5;
  T tl12 = val6i * eqmc6;
  T tl13 = val7i * eqmc7;
  T tl14 = val8i * eqmc8;
  T tl15 = val9i * eqmc9;
  T tl16 = -coef4i * eqmc10;
  T tl17 = -coef4i * eqmc11;
  T tl18 = -coef4i * eqmc12;
  T tl19 = coef3i * eqmc13;
  T tl20 = coef3i * eqmc14;
  T tl21 = coef3i * eqmc15;

  f9[0] = tl1 - T(30.0) * val2i * eqmc1 + val8 * val3i * eqmc2;
  T suma = tl1 + tl2 + tl4;
  T sumb = tl1 + tl3 + tl5;
  T sumc = tl6 + coef4 * tl7;
  T sumd = coef5 * tl12 + coef4 * tl13;
  T sume = tl8 + coef4 * tl9;
  T sumf = -tl12 + coef5 * tl13 + tl14 - coef5 * tl15;
  T sumg = tl10 + coef4 * tl11;
  T sumh = -tl12 + coef5 * tl13 - tl14 + coef5 * tl15;
  T sumi = tl12 + tl13 + tl14 + tl15;
  T sumk = tl12 + tl13 - tl14 - tl15;
  T sump = -coef5 * tl12 - coef5 * tl13;
  T sum67 = tl6 + tl7, sum89 = tl8 + tl9, sum1011 = tl10 + tl11;

  f9[1] = suma + sumc + sumd;
  f9[2] = suma - sumc + sumd;
  f9[3] = suma + sume + sumf;
  f9[4] = suma - sume + sumf;
  f9[5] = suma + sumg + sumh;
  f9[6] = suma - sumg + sumh;
  f9[7] = sumb + sum67 + sum89 + sumi + tl16 + tl19 - tl20;
  f9[8] = sumb - sum67 + sum89 + sumi - tl16 - tl19 - tl20;
  f9[9] = sumb + sum67 - sum89 + sumi - tl16 + tl19 + tl20;
  f9[10] = sumb - sum67 - sum89 + sumi + tl16 - tl19 + tl20;
  f9[11] = sumb + sum67 + sum1011 + sumk + tl18 - tl19 + tl21;
  f9[12] = sumb - sum67 + sum1011 + sumk - tl18 + tl19 + tl21;
  f9[13] = sumb + sum67 - sum1011 + sumk - tl18 - tl19 - tl21;
  f9[14] = sumb - sum67 - sum1011 + sumk + tl18 + tl19 - tl21;
  f9[15] = sumb + sum89 + sum1011 + sump + tl17 + tl20 - tl21;
  f9[16] = sumb - sum89 + sum1011 + sump - tl17 - tl20 - tl21;
  f9[17] = sumb + sum89 - sum1011 + sump - tl17 + tl20 + tl21;
  f9[18] = sumb - sum89 - sum1011 + sump + tl17 - tl20 + tl21;

#pragma unroll
  for (int ip = 0; ip < NPOP; ++ip) f[ip] = f9[ip] + T(0.5) * Fbar[ip];
}

// macrovar's fluid-node branch, B/collision.f90:249-271 (u without force)
template <typename T>
__device__ __forceinline__ void moments(const T (&f9)[NPOP], T& rho9, T& ux9, T& uy9, T& uz9) {
  T sum1 = f9[7] - f9[10], sum2 = f9[9] - f9[8];
  T sum3 = f9[11] - f9[14], sum4 = f9[13] - f9[12];
  T sum5 = f9[15] - f9[18], sum6 = f9[17] - f9[16];
  ux9 = f9[1] - f9[2] + sum1 + sum2 + sum3 + sum4;
  uy9 = f9[3] - f9[4] + sum1 - sum2 + sum5 + sum6;
  uz9 = f9[5] - f9[6] + sum3 - sum4 + sum5 - sum6;
  rho9 = f9[0] + f9[1] + f9[2] + f9[3] + f9[4] + f9[5] + f9[6] + f9[7] + f9[8] + f9[9] +
         f9[10] + f9[11] + f9[12] + f9[13] + f9[14] + f9[15] + f9[16] + f9[17] + f9[18];
}

// body force at node (x, y, z); see ForceView
template <typename T>
__device__ __forceinline__ void body_force(const ForceView<T>& fv, const Geometry& g, int x,
                                           int y, int z, T& fx, T& fy, T& fz) {
  if (fv.mode == FM_CONST) { fx = fv.cfx; fy = fv.cfy; fz = fv.cfz; return; }
  if (fv.mode != FM_TABLE) { fx = T(0); fy = T(0); fz = T(0); return; }
  const T c1 = fv.xtw[4 * x], s1 = fv.xtw[4 * x + 1], c2 = fv.xtw[4 * x + 2], s2 = fv.xtw[4 * x + 3];
  T out[3];
  const T* k = fv.rowtab + ((long long)z * g.ny + y) * kRowCoef;
#pragma unroll
  for (int c = 0; c < 3; ++c)
    out[c] = k[5 * c] + k[5 * c + 1] * c1 + k[5 * c + 2] * s1 + k[5 * c + 3] * c2 + k[5 * c + 4] * s2;
  fx = out[0]; fy = out[1]; fz = out[2];
}

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }




// --------------------------------------------------------------------------
// fused stream + collide (push).  One thread per node, a block covers part
// of an x-row; grid (ceil(nx/B), ny, nz).  Node indices fit in 32 bits
// (N < 2^26 is enforced at context creation).
// FX (FP64 only): collide with exact fixed-point moment sums (collide_fx),
// falling back to collide_fast for the nodes it declines.
// fcache (FX only; fcache_mode 0: unused): the body force per node, three
// component planes of N.  Mode 1 evaluates both fields from their tables;
// mode 2 reads the previous step's field from the cache, which the previous
// launch of this kernel wrote from the same table.  Modes 1 and 2 store this
// step's field at every node (solid ones too: a node that becomes fluid
// reads it next step).
template <typename T, bool CHANNEL, bool FX = false>
__global__ void __launch_bounds__(128, FX ? 4 : 1) k_fused(Geometry g, RatesT<T> r, const T* __restrict__ fin,
                                               T* __restrict__ fout,
                                               const int32_t* __restrict__ isnodes,
                                               ForceView<T> fprev, ForceView<T> fnew,
                                               T* fcache, int fcache_mode) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  const int nx = g.nx, nxy = g.nx * g.ny, N = (int)g.N;
  const int n = x + nx * y + nxy * z;
  T f[NPOP];
  T fp[3];
  // the cached force is loaded with the populations (same latency)
  if constexpr (FX) {
    if (fcache_mode == 2) {
#pragma unroll
      for (int c = 0; c < 3; ++c) fp[c] = fcache[(size_t)c * N + n];
    }
  }
#pragma unroll
  for (int q = 0; q < NPOP; ++q) f[q] = fin[(size_t)q * N + n];
  const bool solid = is_solid(solid_mask(isnodes, g), g, z * g.ny + y, x);
  bool cached = false;
  if constexpr (FX) {
   if (fcache_mode != 0) {
    cached = true;
    T fc[3];
    body_force(fnew, g, x, y, z, fc[0], fc[1], fc[2]);
    if (!solid && fcache_mode != 2) body_force(fprev, g, x, y, z, fp[0], fp[1], fp[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) fcache[(size_t)c * N + n] = fc[c];
    if (!solid) {
      if (!collide_fx(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r)) {
#pragma unroll
        for (int q = 0; q < NPOP; ++q) f[q] = fin[(size_t)q * N + n];
        collide_fast(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
      }
    }
   }
  }
  if (!cached && !solid) {
    T fc[3];
    body_force2(fprev, fnew, x, z * g.ny + y, fp, fc);
    bool done = false;
    if constexpr (FX) {
      done = collide_fx(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
      if (!done) {
        // reloaded rather than kept, so the inputs need no registers
        // during the fixed-point collision
#pragma unroll
        for (int q = 0; q < NPOP; ++q) f[q] = fin[(size_t)q * N + n];
      }
    }
    if (!done) collide_fast(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
  }
  // push: neighbour offsets with periodic wrap
  const int oxp = (x == nx - 1) ? 1 - nx : 1, oxm = (x == 0) ? nx - 1 : -1;
  const int oyp = (y == g.ny - 1) ? nx - nxy : nx, oym = (y == 0) ? nxy - nx : -nx;
  const int ozp = (z == g.nz - 1) ? nxy - N : nxy, ozm = (z == 0) ? N - nxy : -nxy;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) {
    const int cx = cix(q), cy = ciy(q), cz = ciz(q);
    if (CHANNEL && ((cx == -1 && x == 0) || (cx == 1 && x == nx - 1))) {
      // halfway bounce-back at the wall: the outgoing population returns
      // reversed at the same node (C/streaming.f90:175-187)
      fout[(size_t)ipopp(q) * N + n] = f[q];
      continue;
    }
    const int off = (cx > 0 ? oxp : (cx < 0 ? oxm : 0)) + (cy > 0 ? oyp : (cy < 0 ? oym : 0)) +
                    (cz > 0 ? ozp : (cz < 0 ? ozm : 0));
    fout[(size_t)q * N + (n + off)] = f[q];
  }
}

// The body force of a view as fixed point at 2^-kFxF.  Table mode: the row's
// x series with exact 128-bit products of the fixed-point coefficients
// (2^-kFxF, |k| < 2^-7) and twiddles (2^-kTwFix), rounded once; on this GPU
// the integer products run on otherwise idle pipes while FP64 issues at a
// few lanes per clock.
__device__ __forceinline__ void body_force_fx(const ForceView<double>& fv, const Geometry& g, int x,
                                              int y, int z, long long (&o)[3]) {
  if (fv.mode != FM_TABLE) {
    int e = 0;
    const bool cst = fv.mode == FM_CONST;
    o[0] = cst ? fx_from<kFxF>(fv.cfx, e) : 0;
    o[1] = cst ? fx_from<kFxF>(fv.cfy, e) : 0;
    o[2] = cst ? fx_from<kFxF>(fv.cfz, e) : 0;
    return;
  }
  const long long* t = fv.xtw_i + 4 * x;
  const long long c1 = t[0], s1 = t[1], c2 = t[2], s2 = t[3];
  const long long* k = fv.rowtab_i + ((long long)z * g.ny + y) * kRowCoef;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // |products| < 2^124, the sum of five < 2^127
    const __int128 a = (__int128)k[5 * c] * ((__int128)1 << kTwFix) + (__int128)k[5 * c + 1] * c1 +
                       (__int128)k[5 * c + 2] * s1 + (__int128)k[5 * c + 3] * c2 +
                       (__int128)k[5 * c + 4] * s2;
    o[c] = (long long)((a + ((__int128)1 << (kTwFix - 1))) >> kTwFix);
  }
}

// a population read once per step: not kept in L1, which holds the kernel's
// spilled registers and the force tables
__device__ __forceinline__ long long ld_once(const long long* p) {
  long long v;
  asm("ld.global.nc.L1::no_allocate.b64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

// The body force as body_force evaluates it in FP64 (the series of the row
// table, as k_macrovar takes it), then in fixed point at 2^-kFxF: beside the
// all-integer collision core, which leaves the FP64 pipe idle, this costs less
// issue than body_force_fx's twelve 128-bit products.  |F| >= 2^-7 (outside
// the fixed point) raises LBM_ERR_STATE.
__device__ __forceinline__ void body_force_fxd(const ForceView<double>& fv, const Geometry& g,
                                               int x, int y, int z, long long (&o)[3],
                                               DevStatus* st, int n) {
  double v[3];
  body_force(fv, g, x, y, z, v[0], v[1], v[2]);
  int e = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) o[c] = fx_from<kFxF>(v[c], e);
  if (e >= 1023 + (63 - kFxF)) raise_error(st, LBM_ERR_STATE, n);
}

// k_fused's FX path on populations stored in fixed point (collide_fx_fixed):
// the FP64 plain path's kernel between fused steps.  Loads and stores are the
// 64-bit integers themselves; a node collide_fx_fixed declines is converted
// to FP64, collided by collide_fast and converted back (a value beyond the
// fixed-point range, |f| >= 32 or not finite, raises LBM_ERR_NONFINITE).
// The body forces are fixed point too (INTCORE: the series in FP64, rounded
// once, body_force_fxd; otherwise exact integer products, body_force_fx): the
// previous step's enters the velocity as an exact integer add; the force
// cache (fcache_mode as in k_fused) holds them as 64-bit integers at 2^-kFxF.
// CTAs of 128 threads per SM: four with the integer core (128 registers;
// with the force series on the FP64 pipe 3.4 % faster at 256^3 than five at
// 96 registers, twice the spills, and 2.6 % faster than three at 168, no
// spills); five with the FP64-product core (96 registers, 3 % faster than
// four there).
template <bool CHANNEL, bool INTCORE>
__global__ void __launch_bounds__(128, INTCORE ? 4 : 5) k_fused_fixed(Geometry g, RatesT<double> r,
                                                         const long long* __restrict__ fin,
                                                         long long* __restrict__ fout,
                                                         const int32_t* __restrict__ isnodes,
                                                         ForceView<double> fprev,
                                                         ForceView<double> fnew,
                                                         long long* fcache, int fcache_mode,
                                                         DevStatus* st) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  const int nx = g.nx, nxy = g.nx * g.ny, N = (int)g.N;
  const int n = x + nx * y + nxy * z;
  long long f[NPOP];
  long long fp[3], fc[3];
  if (fcache_mode == 2) {
#pragma unroll
    for (int c = 0; c < 3; ++c) fp[c] = fcache[(size_t)c * N + n];
  }
#pragma unroll
  for (int q = 0; q < NPOP; ++q) f[q] = ld_once(fin + (size_t)q * N + n);
  const bool solid = is_solid(solid_mask(isnodes, g), g, z * g.ny + y, x);
  auto force = [&](const ForceView<double>& fv, long long (&o)[3]) {
    if constexpr (INTCORE) body_force_fxd(fv, g, x, y, z, o, st, n);
    else body_force_fx(fv, g, x, y, z, o);
  };
  if (fcache_mode != 0) {
    force(fnew, fc);
    if (!solid && fcache_mode != 2) force(fprev, fp);
#pragma unroll
    for (int c = 0; c < 3; ++c) fcache[(size_t)c * N + n] = fc[c];
  } else if (!solid) {
    force(fprev, fp);
    force(fnew, fc);
  }
  if (!solid) {
    bool done;
    if constexpr (INTCORE) {
      done = collide_fx_fixed_int(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
    } else {
      done = collide_fx_fixed<long long>(f, fp[0], fp[1], fp[2], fx_to<kFxF>(fc[0]),
                                         fx_to<kFxF>(fc[1]), fx_to<kFxF>(fc[2]), r);
    }
    if (!done) {
      const double fx = fx_to<kFxF>(fc[0]), fy = fx_to<kFxF>(fc[1]), fz = fx_to<kFxF>(fc[2]);
      double d[NPOP];
#pragma unroll
      for (int q = 0; q < NPOP; ++q) d[q] = pop_from_fixed(fin[(size_t)q * N + n]);
      collide_fast(d, fx_to<kFxF>(fp[0]), fx_to<kFxF>(fp[1]), fx_to<kFxF>(fp[2]), fx, fy, fz, r);
      bool ok = true;
#pragma unroll
      for (int q = 0; q < NPOP; ++q) ok &= pop_to_fixed(d[q], f[q]);
      if (!ok) raise_error(st, LBM_ERR_NONFINITE, n);
    }
  }
  const int oxp = (x == nx - 1) ? 1 - nx : 1, oxm = (x == 0) ? nx - 1 : -1;
  const int oyp = (y == g.ny - 1) ? nx - nxy : nx, oym = (y == 0) ? nxy - nx : -nx;
  const int ozp = (z == g.nz - 1) ? nxy - N : nxy, ozm = (z == 0) ? N - nxy : -nxy;
#pragma unroll
  for (int q = 0; q < NPOP; ++q) {
    const int cx = cix(q), cy = ciy(q), cz = ciz(q);
    if (CHANNEL && ((cx == -1 && x == 0) || (cx == 1 && x == nx - 1))) {
      fout[(size_t)ipopp(q) * N + n] = f[q];
      continue;
    }
    const int off = (cx > 0 ? oxp : (cx < 0 ? oxm : 0)) + (cy > 0 ? oyp : (cy < 0 ? oym : 0)) +
                    (cz > 0 ? ozp : (cz < 0 ? ozm : 0));
    fout[(size_t)q * N + (n + off)] = f[q];
  }
}

// the stored populations between FP64 and fixed point, in place
__global__ void k_pop_to_fixed(double* f, long long n, DevStatus* st) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long v;
    if (!pop_to_fixed(f[i], v)) raise_error(st, LBM_ERR_NONFINITE, (int)(i % 2147483647));
    reinterpret_cast<long long*>(f)[i] = v;
  }
}
__global__ void k_pop_from_fixed(double* f, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    f[i] = pop_from_fixed(reinterpret_cast<const long long*>(f)[i]);
}

// streaming alone (per-subroutine entry), B/streaming.f90:2-171
template <typename T, bool CHANNEL>
__global__ void k_stream(Geometry g, const T* __restrict__ fin, T* __restrict__ fout) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  const long long N = g.N;
  const long long n = x + (long long)g.nx * (y + (long long)g.ny * z);
  fout[n] = fin[n];
#pragma unroll
  for (int q = 1; q < NPOP; ++q) {
    int cx = cix(q), cy = ciy(q), cz = ciz(q);
    T v = fin[q * N + n];
    if (CHANNEL && ((cx == -1 && x == 0) || (cx == 1 && x == g.nx - 1))) {
      fout[ipopp(q) * N + n] = v;
      continue;
    }
    int xd = wrapi(x + cx, g.nx), yd = wrapi(y + cy, g.ny), zd = wrapi(z + cz, g.nz);
    fout[q * N + xd + (long long)g.nx * (yd + (long long)g.ny * zd)] = v;
  }
}

// collision_MRT alone (per-subroutine entry), in place, using the stored
// macroscopic arrays as the reference does
template <typename T>
__global__ void k_collision(Geometry g, Rates r, T* __restrict__ f,
                            const int32_t* __restrict__ isnodes, ForceView<T> fv,
                            const T* __restrict__ rho, const T* __restrict__ ux,
                            const T* __restrict__ uy, const T* __restrict__ uz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  const long long N = g.N;
  const long long n = x + (long long)g.nx * (y + (long long)g.ny * z);
  if (isnodes[n] >= 0) return;
  T fl[NPOP];
#pragma unroll
  for (int q = 0; q < NPOP; ++q) fl[q] = f[q * N + n];
  T fx, fy, fz;
  body_force(fv, g, x, y, z, fx, fy, fz);
  collide_mrt(fl, rho[n], ux[n], uy[n], uz[n], fx, fy, fz, r);
#pragma unroll
  for (int q = 0; q < NPOP; ++q) f[q * N + n] = fl[q];
}

// macrovar, B/collision.f90:232-332 (solid branch with nearest image; the
// channel has no x image, C/collision.f90:294-295)
template <typename T>
__global__ void k_macrovar(Geometry g, const T* __restrict__ f,
                           const int32_t* __restrict__ isnodes, ForceView<T> fv,
                           ParticleView pv, T* __restrict__ rho, T* __restrict__ ux,
                           T* __restrict__ uy, T* __restrict__ uz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  const long long N = g.N;
  const long long n = x + (long long)g.nx * (y + (long long)g.ny * z);
  T fl[NPOP];
#pragma unroll
  for (int q = 0; q < NPOP; ++q) fl[q] = f[q * N + n];
  T rho9, ux9, uy9, uz9, fx, fy, fz;
  moments(fl, rho9, ux9, uy9, uz9);
  body_force(fv, g, x, y, z, fx, fy, fz);
  T u1 = ux9 + fx * T(0.5), u2 = uy9 + fy * T(0.5), u3 = uz9 + fz * T(0.5), rr = rho9;
  int id = isnodes[n];
  if (id >= 0 && pv.ypglb != nullptr) {
    double xpnt = (double)(x + 1) - 0.5, ypnt = (double)(y + 1) - 0.5, zpnt = (double)(z + 1) - 0.5;
    double xc = pv.ypglb[3 * id], yc = pv.ypglb[3 * id + 1], zc = pv.ypglb[3 * id + 2];
    if (!g.channel) {
      if ((xc - xpnt) > (double)g.nxh) xc = xc - (double)g.nx;
      if ((xc - xpnt) < -(double)g.nxh) xc = xc + (double)g.nx;
    }
    if ((yc - ypnt) > (double)g.nyh) yc = yc - (double)g.ny;
    if ((yc - ypnt) < -(double)g.nyh) yc = yc + (double)g.ny;
    if ((zc - zpnt) > (double)g.nzh) zc = zc - (double)g.nz;
    if ((zc - zpnt) < -(double)g.nzh) zc = zc + (double)g.nz;
    double xx0 = xpnt - xc, yy0 = ypnt - yc, zz0 = zpnt - zc;
    const double* w = pv.wp + 3 * id;
    const double* o = pv.omgp + 3 * id;
    u1 = T(w[0] + (o[1] * zz0 - o[2] * yy0));
    u2 = T(w[1] + (o[2] * xx0 - o[0] * zz0));
    u3 = T(w[2] + (o[0] * yy0 - o[1] * xx0));
    rr = T(pv.rhopart);
  }
  rho[n] = rr; ux[n] = u1; uy[n] = u2; uz[n] = u3;
}

template <typename T>
__global__ void k_rhoupdat(Geometry g, const T* __restrict__ f, T* __restrict__ rho) {
  long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  T r = f[n];
#pragma unroll
  for (int q = 1; q < NPOP; ++q) r = r + f[q * g.N + n];
  rho[n] = r;
}

// rhoupdat that also reports max |rho_new - rho_old| (the pre-relaxation
// test of B/main.f90:91-93) through an atomic max on the bits of the
// non-negative FP64 difference (ordered like the values)
template <typename T>
__global__ void __launch_bounds__(256) k_rhoupdat_maxdiff(Geometry g, const T* __restrict__ f,
                                                          T* __restrict__ rho,
                                                          unsigned long long* maxbits) {
  long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double d = 0.0;
  if (n < g.N) {
    T r = f[n];
#pragma unroll
    for (int q = 1; q < NPOP; ++q) r = r + f[q * g.N + n];
    d = fabs((double)r - (double)rho[n]);
    if (!(d == d)) d = __longlong_as_double(0x7ff0000000000000LL);  // NaN -> +inf
    rho[n] = r;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
  __shared__ double wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = wm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, wm[w]);
    atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
  }
}

// initpop, B/initial.f90:14-26 (rho' = 0)
template <typename T>
__global__ void k_initpop(Geometry g, const double* __restrict__ ux, const double* __restrict__ uy,
                          const double* __restrict__ uz, T* __restrict__ f, T* __restrict__ rho) {
  long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  double u1 = ux[n], u2 = uy[n], u3 = uz[n];
  double usqr = u1 * u1 + u2 * u2 + u3 * u3;
  usqr = 1.5 * usqr;
  const double r0 = 0.0;
  f[n] = T((1.0 / 3.0) * (r0 - usqr));
#pragma unroll
  for (int q = 1; q < NPOP; ++q) {
    double G = cix(q) * u1 + ciy(q) * u2 + ciz(q) * u3;
    double w = q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0;
    f[q * g.N + n] = T(w * (r0 + 3.0 * G + 4.5 * G * G - usqr));
  }
  rho[n] = T(0);
}

// Fortran-order f(0:18, lx, ly, lz) chunk <-> structure of arrays
template <typename T>
__global__ void k_aos_to_soa(Geometry g, const double* __restrict__ aos, T* __restrict__ soa,
                             long long node0, long long nnodes) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nnodes * NPOP) return;
  long long nl = t / NPOP;
  int q = (int)(t - nl * NPOP);
  soa[q * g.N + node0 + nl] = T(aos[t]);
}
template <typename T>
__global__ void k_soa_to_aos(Geometry g, const T* __restrict__ soa, double* __restrict__ aos,
                             long long node0, long long nnodes) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nnodes * NPOP) return;
  long long nl = t / NPOP;
  int q = (int)(t - nl * NPOP);
  aos[t] = (double)soa[q * g.N + node0 + nl];
}
// Host transfers of the reference-layout populations f(0:18, x, y, z) that
// read or write page-locked host memory directly over the CPU-GPU link (no
// staging copy): a block moves tiles of kXTile nodes, the AoS side as one
// contiguous run with 16-byte accesses, transposed in shared memory, the SoA
// side as coalesced rows.
constexpr int kXTile = 256;
template <typename T>
__global__ void __launch_bounds__(256) k_aos_host_to_soa(const double* __restrict__ aos,
                                                         T* __restrict__ soa, long long N) {
  extern __shared__ double tile[];
  const long long ntiles = (N + kXTile - 1) / kXTile;
  for (long long ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const long long a0 = ti * kXTile;
    const int nn = (int)min((long long)kXTile, N - a0);
    const double* src = aos + a0 * NPOP;
    const int total = nn * NPOP;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
      const double2* s2 = reinterpret_cast<const double2*>(src);
      for (int i = threadIdx.x; i < (total >> 1); i += blockDim.x) {
        const double2 v = s2[i];
        tile[2 * i] = v.x;
        tile[2 * i + 1] = v.y;
      }
      if ((total & 1) && threadIdx.x == 0) tile[total - 1] = src[total - 1];
    } else {
      for (int i = threadIdx.x; i < total; i += blockDim.x) tile[i] = src[i];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int q = i / nn, n = i - q * nn;
      soa[(long long)q * N + a0 + n] = T(tile[n * NPOP + q]);
    }
    __syncthreads();
  }
}
// FIXED: soa holds the 64-bit fixed-point populations of the FP64 plain path
// (g.pop_fixed), converted here on the way out rather than in place first
template <typename T, bool FIXED = false>
__global__ void __launch_bounds__(256) k_soa_to_aos_host(const T* __restrict__ soa,
                                                         double* __restrict__ aos, long long N) {
  extern __shared__ double tile[];
  const long long ntiles = (N + kXTile - 1) / kXTile;
  for (long long ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const long long a0 = ti * kXTile;
    const int nn = (int)min((long long)kXTile, N - a0);
    double* dst = aos + a0 * NPOP;
    const int total = nn * NPOP;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int q = i / nn, n = i - q * nn;
      if constexpr (FIXED)
        tile[n * NPOP + q] = pop_from_fixed(soa[(long long)q * N + a0 + n]);
      else
        tile[n * NPOP + q] = (double)soa[(long long)q * N + a0 + n];
    }
    __syncthreads();
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
      double2* d2 = reinterpret_cast<double2*>(dst);
      for (int i = threadIdx.x; i < (total >> 1); i += blockDim.x)
        d2[i] = make_double2(tile[2 * i], tile[2 * i + 1]);
      if ((total & 1) && threadIdx.x == 0) dst[total - 1] = tile[total - 1];
    } else {
      for (int i = threadIdx.x; i < total; i += blockDim.x) dst[i] = tile[i];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void k_convert(const double* __restrict__ in, T* __restrict__ out, long long n) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = T(in[t]);
}
template <typename T>
__global__ void k_convert_back(const T* __restrict__ in, double* __restrict__ out, long long n) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = (double)in[t];
}

template <typename T>
__global__ void k_force_field(Geometry g, ForceView<T> fv, double* fx, double* fy, double* fz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= g.nx) return;
  long long n = x + (long long)g.nx * (y + (long long)g.ny * z);
  T a, b, c;
  body_force(fv, g, x, y, z, a, b, c);
  fx[n] = (double)a; fy[n] = (double)b; fz[n] = (double)c;
}

// FP64 mass and momentum partial sums, one value set per block
template <typename T>
__global__ void k_mass_momentum(Geometry g, const T* __restrict__ f, double* partial) {
  double m[4] = {0, 0, 0, 0};
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.N;
       n += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < NPOP; ++q) {
      double v = (double)f[q * g.N + n];
      m[0] += v;
      m[1] += cix(q) * v;
      m[2] += ciy(q) * v;
      m[3] += ciz(q) * v;
    }
  }
  __shared__ double sm[4][256];
#pragma unroll
  for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] = m[c];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 4; ++c) partial[4 * blockIdx.x + c] = sm[c][0];
}

// Forcing tables.  Stage 1 (ztab): A(c, kx, jy, z) = sum_kz a(c,kx,jy,kz)
// exp(+2 pi i kz z / nz); stage 2 (rowtab): B(c, kx, z, y) = sum_jy A
// exp(+2 pi i ky y / ny).  Together with the per-x twiddles they evaluate
// the inverse transform of gaussian.f90:557-601 at any node.
template <typename ZT>
__device__ __forceinline__ void k_force_ztab_body(int bx, int gx, Geometry g, const ForcingDev* st, const double* __restrict__ ztw,
                             ZT* ztab) {
  int t = bx * blockDim.x + threadIdx.x;  // over (c, kx, jy, z)
  int total = 3 * 3 * 5 * g.nz;
  if (t >= total) return;
  int z = t % g.nz;
  int r = t / g.nz;
  int jy = r % 5; r /= 5;
  int kx = r % 3;
  int c = r / 3;
  const double* a = st->a + 150 * c;
  double sr = 0.0, si = 0.0;
  for (int kz = 0; kz < 5; ++kz) {
    double cr = a[(2 * kx) + 6 * jy + 30 * kz];
    double ci = a[(2 * kx + 1) + 6 * jy + 30 * kz];
    double cs = ztw[2 * (kz * g.nz + z)], sn = ztw[2 * (kz * g.nz + z) + 1];
    sr += cr * cs - ci * sn;
    si += cr * sn + ci * cs;
  }
  // stored in the table's precision (the row sums read it without conversion)
  ztab[2 * t] = ZT(sr);
  ztab[2 * t + 1] = ZT(si);
}
template <typename ZT>
__global__ void k_force_ztab(Geometry g, const ForcingDev* st, const double* __restrict__ ztw,
                             ZT* ztab) {
  k_force_ztab_body<ZT>(blockIdx.x, gridDim.x, g, st, ztw, ztab);
}

// Row coefficients of the force series (kRowCoef layout) from the (kx, z)
// table: one thread per (row, component, kx).  The kx = 1, 2 terms of the
// real inverse transform enter twice (kx and -kx), hence the factor 2.
template <typename T>
__device__ __forceinline__ void k_force_rowtab_body(int bx, int gx, Geometry g, const T* __restrict__ ztab,
                               const T* __restrict__ ytw, T* __restrict__ rowtab,
                               long long* rowtab_i = nullptr, DevStatus* status = nullptr) {
  long long t = bx * (long long)blockDim.x + threadIdx.x;  // over (c,kx,z,y)
  long long total = 9LL * g.nz * g.ny;
  if (t >= total) return;
  int y = (int)(t % g.ny);
  long long r = t / g.ny;
  int z = (int)(r % g.nz);
  int ckx = (int)(r / g.nz);
  T sr = T(0), si = T(0);
#pragma unroll
  for (int jy = 0; jy < 5; ++jy) {
    long long ai = ((long long)(ckx * 5 + jy)) * g.nz + z;
    T ar = ztab[2 * ai], aim = ztab[2 * ai + 1];
    T cs = ytw[2 * (jy * g.ny + y)], sn = ytw[2 * (jy * g.ny + y) + 1];
    sr += ar * cs - aim * sn;
    si += ar * sn + aim * cs;
  }
  const int c = ckx / 3, kx = ckx % 3;
  const long long row = ((long long)z * g.ny + y) * kRowCoef;
  T* k = rowtab + row + 5 * c;
  T v0, v1 = T(0);
  int j0;
  if (kx == 0) {
    k[0] = v0 = sr;
    j0 = 0;
    if (c == 0) rowtab[row + 15] = T(0);
  } else {
    k[2 * kx - 1] = v0 = T(2.0) * sr;
    k[2 * kx] = v1 = T(-2.0) * si;
    j0 = 2 * kx - 1;
  }
  if constexpr (sizeof(T) == 8) {
    if (rowtab_i) {
      // fixed point at 2^-kFxF: exact for |k| >= 2^-(kFxF - 52), range |k| < 2^-7
      long long* ki = rowtab_i + row + 5 * c;
      int e = 0;
      ki[j0] = fx_from<kFxF>(double(v0), e);
      if (kx != 0) ki[j0 + 1] = fx_from<kFxF>(double(v1), e);
      if (kx == 0 && c == 0) rowtab_i[row + 15] = 0;
      if (e >= 1023 + (63 - kFxF)) raise_error(status, LBM_ERR_STATE, (int)(t % 2147483647));
    }
  }
}
template <typename T>
__global__ void k_force_rowtab(Geometry g, const T* __restrict__ ztab,
                               const T* __restrict__ ytw, T* __restrict__ rowtab,
                               long long* rowtab_i, DevStatus* status) {
  k_force_rowtab_body<T>(blockIdx.x, gridDim.x, g, ztab, ytw, rowtab, rowtab_i, status);
}

inline dim3 row_grid(const Geometry& g, int bx) { return dim3((g.nx + bx - 1) / bx, g.ny, g.nz); }
inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
template <typename T>
void launch_fused_step(const Geometry& g, const Rates& r, const T* fin, T* fout,
                       const int32_t* isnodes, const ForceView<T>& fprev,
                       const ForceView<T>& fnew, bool fx, T* fcache, int fcache_mode,
                       cudaStream_t s) {
  const int B = 128;
  const RatesT<T> rt = rates_t<T>(r);
  if constexpr (sizeof(T) == 8) {
    if (fx) {
      if (!fcache || fnew.mode != FM_TABLE) fcache_mode = 0;
      if (g.channel)
        k_fused<T, true, true><<<row_grid(g, B), B, 0, s>>>(g, rt, fin, fout, isnodes, fprev, fnew,
                                                            fcache, fcache_mode);
      else
        k_fused<T, false, true><<<row_grid(g, B), B, 0, s>>>(g, rt, fin, fout, isnodes, fprev, fnew,
                                                             fcache, fcache_mode);
      count_launch();
      return;
    }
  }
  if (g.channel)
    { k_fused<T, true><<<row_grid(g, B), B, 0, s>>>(g, rt, fin, fout, isnodes, fprev, fnew, nullptr, 0); count_launch(); }
  else
    { k_fused<T, false><<<row_grid(g, B), B, 0, s>>>(g, rt, fin, fout, isnodes, fprev, fnew, nullptr, 0); count_launch(); }
}

void launch_fused_fixed(const Geometry& g, const Rates& r, bool int_core, const double* fin,
                        double* fout, const int32_t* isnodes, const ForceView<double>& fprev,
                        const ForceView<double>& fnew, double* fcache, int fcache_mode,
                        DevStatus* st, cudaStream_t s) {
  const int B = 128;
  const RatesT<double> rt = rates_t<double>(r);
  if (!fcache || fnew.mode != FM_TABLE) fcache_mode = 0;
  const long long* gi = reinterpret_cast<const long long*>(fin);
  long long* go = reinterpret_cast<long long*>(fout);
  long long* fci = reinterpret_cast<long long*>(fcache);
  auto launch = [&](auto kern) {
    kern<<<row_grid(g, B), B, 0, s>>>(g, rt, gi, go, isnodes, fprev, fnew, fci, fcache_mode, st);
  };
  if (int_core)
    g.channel ? launch(k_fused_fixed<true, true>) : launch(k_fused_fixed<false, true>);
  else
    g.channel ? launch(k_fused_fixed<true, false>) : launch(k_fused_fixed<false, false>);
  count_launch();
}

void launch_pop_format(double* f, long long n, bool to_fixed, DevStatus* st, cudaStream_t s) {
  const int B = 256;
  long long blocks = (n + B - 1) / B;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (to_fixed) k_pop_to_fixed<<<(unsigned)blocks, B, 0, s>>>(f, n, st);
  else k_pop_from_fixed<<<(unsigned)blocks, B, 0, s>>>(f, n);
  count_launch();
}

template <typename T>
void launch_macrovar(const Geometry& g, const T* f, const int32_t* isnodes,
                     const ForceView<T>& fv, const ParticleView& pv, T* rho, T* ux, T* uy,
                     T* uz, cudaStream_t s) {
  { k_macrovar<T><<<row_grid(g, 128), 128, 0, s>>>(g, f, isnodes, fv, pv, rho, ux, uy, uz); count_launch(); }
}

template <typename T>
void launch_collision(const Geometry& g, const Rates& r, T* f, const int32_t* isnodes,
                      const ForceView<T>& fv, const T* rho, const T* ux, const T* uy,
                      const T* uz, cudaStream_t s) {
  { k_collision<T><<<row_grid(g, 128), 128, 0, s>>>(g, r, f, isnodes, fv, rho, ux, uy, uz); count_launch(); }
}

template <typename T>
void launch_streaming(const Geometry& g, const T* fin, T* fout, cudaStream_t s) {
  if (g.channel)
    { k_stream<T, true><<<row_grid(g, 128), 128, 0, s>>>(g, fin, fout); count_launch(); }
  else
    { k_stream<T, false><<<row_grid(g, 128), 128, 0, s>>>(g, fin, fout); count_launch(); }
}

template <typename T>
void launch_rhoupdat_maxdiff(const Geometry& g, const T* f, T* rho, unsigned long long* maxbits,
                             cudaStream_t s) {
  cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), s);
  { k_rhoupdat_maxdiff<T><<<blocks_for(g.N, 256), 256, 0, s>>>(g, f, rho, maxbits); count_launch(); }
}

template <typename T>
void launch_rhoupdat(const Geometry& g, const T* f, T* rho, cudaStream_t s) {
  { k_rhoupdat<T><<<blocks_for(g.N, 256), 256, 0, s>>>(g, f, rho); count_launch(); }
}

template <typename T>
void launch_initpop(const Geometry& g, const double* ux, const double* uy, const double* uz,
                    T* f, T* rho, cudaStream_t s) {
  { k_initpop<T><<<blocks_for(g.N, 256), 256, 0, s>>>(g, ux, uy, uz, f, rho); count_launch(); }
}

template <typename T>
void launch_aos_to_soa(const Geometry& g, const double* aos, T* soa, long long node0,
                       long long nnodes, cudaStream_t s) {
  { k_aos_to_soa<T><<<blocks_for(nnodes * NPOP, 256), 256, 0, s>>>(g, aos, soa, node0, nnodes); count_launch(); }
}
template <typename T>
void launch_soa_to_aos(const Geometry& g, const T* soa, double* aos, long long node0,
                       long long nnodes, cudaStream_t s) {
  { k_soa_to_aos<T><<<blocks_for(nnodes * NPOP, 256), 256, 0, s>>>(g, soa, aos, node0, nnodes); count_launch(); }
}
template <typename T>
void launch_aos_host_to_soa(const double* aos_mapped, T* soa, long long N, int sms,
                            cudaStream_t s) {
  const size_t smem = (size_t)kXTile * NPOP * sizeof(double);
  const long long ntiles = (N + kXTile - 1) / kXTile;
  const unsigned grid = (unsigned)std::min<long long>(ntiles, 5LL * sms);
  { k_aos_host_to_soa<T><<<grid, 256, smem, s>>>(aos_mapped, soa, N); count_launch(); }
}
template <typename T>
void launch_soa_to_aos_host(const T* soa, double* aos_mapped, long long N, int sms,
                            cudaStream_t s) {
  const size_t smem = (size_t)kXTile * NPOP * sizeof(double);
  const long long ntiles = (N + kXTile - 1) / kXTile;
  const unsigned grid = (unsigned)std::min<long long>(ntiles, 5LL * sms);
  { k_soa_to_aos_host<T><<<grid, 256, smem, s>>>(soa, aos_mapped, N); count_launch(); }
}
void launch_soa_fixed_to_aos_host(const long long* soa, double* aos_mapped, long long N, int sms,
                                  cudaStream_t s) {
  const size_t smem = (size_t)kXTile * NPOP * sizeof(double);
  const long long ntiles = (N + kXTile - 1) / kXTile;
  const unsigned grid = (unsigned)std::min<long long>(ntiles, 5LL * sms);
  { k_soa_to_aos_host<long long, true><<<grid, 256, smem, s>>>(soa, aos_mapped, N); count_launch(); }
}
template <typename T>
void launch_convert(const double* in, T* out, long long n, cudaStream_t s) {
  { k_convert<T><<<blocks_for(n, 256), 256, 0, s>>>(in, out, n); count_launch(); }
}
template <typename T>
void launch_convert_back(const T* in, double* out, long long n, cudaStream_t s) {
  { k_convert_back<T><<<blocks_for(n, 256), 256, 0, s>>>(in, out, n); count_launch(); }
}
template <typename T>
void launch_force_field(const Geometry& g, const ForceView<T>& fv, double* fx, double* fy,
                        double* fz, cudaStream_t s) {
  { k_force_field<T><<<row_grid(g, 128), 128, 0, s>>>(g, fv, fx, fy, fz); count_launch(); }
}
template <typename T>
void launch_mass_momentum(const Geometry& g, const T* f, double* partial, int nblocks,
                          cudaStream_t s) {
  { k_mass_momentum<T><<<nblocks, 256, 0, s>>>(g, f, partial); count_launch(); }
}

namespace {
__global__ void k_force_ztab_multi(const BoxForcing* boxes) {
  const BoxForcing& B = boxes[blockIdx.y];
  const int nblk = (45 * B.g.nz + 127) / 128;
  if ((int)blockIdx.x >= nblk) return;
  k_force_ztab_body<float>(blockIdx.x, nblk, B.g, B.st, B.ztw, B.ztab);
}
__global__ void k_force_rowtab_multi(const BoxForcing* boxes, int slot) {
  const BoxForcing& B = boxes[blockIdx.y];
  const long long nblk = (9LL * B.g.nz * B.g.ny + 255) / 256;
  if ((long long)blockIdx.x >= nblk) return;
  k_force_rowtab_body<float>(blockIdx.x, (int)nblk, B.g, B.ztab, B.ytw, B.rowtab[slot]);
}
}  // namespace

void launch_forcing_update_multi(const BoxForcing* boxes, int nb, cudaStream_t s);

void launch_forcing_multi(const BoxForcing* boxes, int nb, int max_nz, long long max_rows,
                          int slot, cudaStream_t s) {
  if (nb <= 0) return;
  launch_forcing_update_multi(boxes, nb, s);
  k_force_ztab_multi<<<dim3((45 * max_nz + 127) / 128, nb), 128, 0, s>>>(boxes);
  count_launch();
  k_force_rowtab_multi<<<dim3((unsigned)((9 * max_rows + 255) / 256), nb), 256, 0, s>>>(boxes, slot);
  count_launch();
}

template <typename T>
void launch_forcing_tables(const Geometry& g, const ForcingDev* st, const T* ytw,
                           const double* ztw, T* rowtab, T* ztab, cudaStream_t s,
                           long long* rowtab_i, DevStatus* status) {
  int nz_t = 45 * g.nz;
  { k_force_ztab<T><<<blocks_for(nz_t, 128), 128, 0, s>>>(g, st, ztw, ztab); count_launch(); }
  long long nr = 9LL * g.nz * g.ny;
  { k_force_rowtab<T><<<blocks_for(nr, 256), 256, 0, s>>>(g, ztab, ytw, rowtab, rowtab_i, status); count_launch(); }
}

#define LBM_INSTANTIATE(T)                                                                   \
  template void launch_fused_step<T>(const Geometry&, const Rates&, const T*, T*,           \
                                     const int32_t*, const ForceView<T>&,                   \
                                     const ForceView<T>&, bool, T*, int, cudaStream_t);     \
  template void launch_macrovar<T>(const Geometry&, const T*, const int32_t*,               \
                                   const ForceView<T>&, const ParticleView&, T*, T*, T*, T*, \
                                   cudaStream_t);                                           \
  template void launch_collision<T>(const Geometry&, const Rates&, T*, const int32_t*,      \
                                    const ForceView<T>&, const T*, const T*, const T*,      \
                                    const T*, cudaStream_t);                                \
  template void launch_streaming<T>(const Geometry&, const T*, T*, cudaStream_t);           \
  template void launch_rhoupdat<T>(const Geometry&, const T*, T*, cudaStream_t);            \
  template void launch_rhoupdat_maxdiff<T>(const Geometry&, const T*, T*, unsigned long long*, \
                                           cudaStream_t);                                      \
  template void launch_initpop<T>(const Geometry&, const double*, const double*,            \
                                  const double*, T*, T*, cudaStream_t);                     \
  template void launch_aos_to_soa<T>(const Geometry&, const double*, T*, long long,         \
                                     long long, cudaStream_t);                              \
  template void launch_soa_to_aos<T>(const Geometry&, const T*, double*, long long,         \
                                     long long, cudaStream_t);                              \
  template void launch_aos_host_to_soa<T>(const double*, T*, long long, int, cudaStream_t);  \
  template void launch_soa_to_aos_host<T>(const T*, double*, long long, int, cudaStream_t);  \
  template void launch_convert<T>(const double*, T*, long long, cudaStream_t);              \
  template void launch_convert_back<T>(const T*, double*, long long, cudaStream_t);         \
  template void launch_force_field<T>(const Geometry&, const ForceView<T>&, double*,        \
                                      double*, double*, cudaStream_t);                      \
  template void launch_mass_momentum<T>(const Geometry&, const T*, double*, int,            \
                                        cudaStream_t);                                      \
  template void launch_forcing_tables<T>(const Geometry&, const ForcingDev*, const T*, \
                                         const double*, T*, T*, cudaStream_t, long long*, \
                                         DevStatus*);

LBM_INSTANTIATE(double)
LBM_INSTANTIATE(float)

}  // namespace lbm
