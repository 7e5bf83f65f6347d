// Host check of the FP64 plain path's collision cores (test infrastructure):
// the all-integer core (collide_fx_fixed_int) against the core with FP64
// velocity and force products (collide_fx_fixed<long long>) on random
// near-equilibrium states, both MRT rate sets.  Prints one line per rate set:
//   mrt max_abs_diff declined_int declined_fp64 declined_by_int_only
//   declined_by_fp64_only states
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "lbm_collide.cuh"

using namespace lbm;

// fx_out_of_range tests |x| >= 2^56 on the high word; the 64-bit form of
// the same test, for comparison
static bool out_of_range_64(long long x) {
  const unsigned long long lim = 1ULL << (kFxOut + kFxOutMax);
  return (unsigned long long)x + lim >= 2 * lim;
}

int main(int argc, char** argv) {
  const int n_states = argc > 1 ? std::atoi(argv[1]) : 100000;
  {
    long long bad = 0, n = 0;
    std::mt19937_64 rng(77);
    const long long lim = 1LL << (kFxOut + kFxOutMax);
    const long long edges[] = {0, 1, -1, lim - 1, lim, lim + 1, -lim + 1, -lim, -lim - 1,
                               (1LL << 62), -(1LL << 62), 0x7fffffffffffffffLL,
                               (long long)0x8000000000000000ULL, lim - (1LL << 32),
                               -lim + (1LL << 32), lim + (1LL << 32) - 1};
    for (long long x : edges) { ++n; bad += (fx_out_of_range(x) != 0) != out_of_range_64(x); }
    for (int i = 0; i < 2000000; ++i) {
      const long long x = (long long)rng() >> (i % 10);
      ++n;
      bad += (fx_out_of_range(x) != 0) != out_of_range_64(x);
    }
    std::printf("range %lld %lld\n", bad, n);
  }
  for (int mrt = 1; mrt <= 2; ++mrt) {
    Rates rr;
    const double tau = 3 * 0.0036 + 0.5;
    rr.s9 = 1.0 / tau;
    rr.s13 = rr.s9;
    if (mrt == 1) {
      rr.s1 = 1.19; rr.s2 = 1.4; rr.s4 = 1.2; rr.s10 = 1.4; rr.s16 = 1.98;
      rr.omegepsl = 0.0; rr.omegepslj = -475.0 / 63.0; rr.omegxx = 0.0;
    } else {
      rr.s1 = rr.s2 = rr.s4 = rr.s10 = rr.s16 = rr.s9;
      rr.omegepsl = 3.0; rr.omegepslj = -5.5; rr.omegxx = -0.5;
    }
    const RatesT<double> r = rates_t<double>(rr);
    std::mt19937_64 rng(1234 + mrt);
    std::normal_distribution<double> nd(0.0, 1.0);
    const double w[19] = {1. / 3,  1. / 18, 1. / 18, 1. / 18, 1. / 18, 1. / 18, 1. / 18,
                          1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36,
                          1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36};
    double maxd = 0.0;
    long long dec_int = 0, dec_fp = 0, int_only = 0, fp_only = 0;
    for (int it = 0; it < n_states; ++it) {
      const double us = (it % 40 == 0) ? 0.3 : 0.05;  // a few states beyond |u| < 1/4
      const double u[3] = {us * nd(rng), us * nd(rng), us * nd(rng)};
      double f[19];
      for (int q = 0; q < 19; ++q) {
        const double cu = cix(q) * u[0] + ciy(q) * u[1] + ciz(q) * u[2];
        f[q] = w[q] * (0.01 * nd(rng) + 3 * cu + 4.5 * cu * cu -
                       1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2])) +
               1e-4 * w[q] * nd(rng);
      }
      const double F[3] = {3e-5 * nd(rng), 3e-5 * nd(rng), 3e-5 * nd(rng)};
      const double Fp[3] = {F[0] * 0.9, F[1] * 1.1, F[2]};
      long long g[19], a[19], b[19];
      int e = 0;
      for (int q = 0; q < 19; ++q) g[q] = fx_from<kFxIn>(f[q], e);
      long long fp[3], fc[3];
      for (int c = 0; c < 3; ++c) {
        fp[c] = fx_from<kFxF>(Fp[c], e);
        fc[c] = fx_from<kFxF>(F[c], e);
      }
      std::memcpy(a, g, sizeof g);
      std::memcpy(b, g, sizeof g);
      const bool ri = collide_fx_fixed_int(a, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
      const bool rf = collide_fx_fixed<long long>(b, fp[0], fp[1], fp[2], fx_to<kFxF>(fc[0]),
                                                  fx_to<kFxF>(fc[1]), fx_to<kFxF>(fc[2]), r);
      dec_int += !ri;
      dec_fp += !rf;
      int_only += (!ri && rf);
      fp_only += (ri && !rf);
      if (ri != rf) continue;
      if (!ri) continue;
      for (int q = 0; q < 19; ++q)
        maxd = std::fmax(maxd, std::fabs((double)(a[q] - b[q])) * std::ldexp(1.0, -kFxIn));
    }
    std::printf("%d %.6e %lld %lld %lld %lld %d\n", mrt, maxd, dec_int, dec_fp, int_only, fp_only,
                n_states);
  }
  return 0;
}
