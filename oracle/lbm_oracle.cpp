// lbm_oracle.cpp - CPU restatement of the reference's particle-laden D3Q19
// MRT lattice Boltzmann time step, used ONLY as test infrastructure: the
// parity tests, the smoke check and the CPU-baseline leg of bench.py compare
// the engine with it.  Nothing in the product library links or calls this file.
//
// Parity status: pinned against the reference's own run.  The reference is
// Fortran 90 + MPI + FFTW 2 with no Fortran compiler on either machine, so
// its hot-path sources are translated to C++ by oracle/fortran and run on one
// process (oracle/refrun.py); tests/test_reference_pin.py holds this
// restatement to that run (the channel program bit for bit, the box program
// bit for bit up to its FFT-synthesised stochastic force, 1e-13), and
// tests/test_reference_golden.py to fixtures recorded from it.  The
// reference ships no tests or golden vectors of its own.
//
// Each routine follows one reference subroutine line by line, for a single
// periodic domain: the MPI halo exchanges become periodic index wraps and the
// MPI_ALLREDUCE sums become plain sums.  Expressions keep the reference's
// evaluation order (Fortran evaluates a+b-c left to right) and the file is
// compiled with -ffp-contract=off, so the integer decisions (solid flags,
// links, bounce-back branches, refill events) are reproducible bit for bit.
//
// Abbreviations in citations: B/ = 3DBox_Forced_HI_Turbulence_Moving_Particles_LBM,
// C/ = 3DChannel_Decaying_HIT_Finite_Size_Moving_Particles.
//
// Layout: all node arrays are 0-based with x fastest, node = i + nx*(j + ny*k)
// (Fortran (i+1, j+1, k+1)); populations are f[ip*N + node] (structure of
// arrays).  Particle ids are 0-based (reference id - 1); particle vectors are
// (3, npart) with the component fastest, as in var_inc.

#include "../include/lbm.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

const int NPOP = 19;
// B/para.f90:171-175
const int CIX[NPOP] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CIY[NPOP] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CIZ[NPOP] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
const int IPOPP[NPOP] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

// Park-Miller minimal standard generator with Bays-Durham shuffle
// (Numerical Recipes ran1), as ranff B/gaussian.f90:374-404 and ranpp
// B/partlib.f90:83-115.  iv is the 32-entry shuffle table (0-based here).
double ran1(int32_t* idum, int32_t* iy, int32_t* iv) {
  const int32_t IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, NTAB = 32;
  const int32_t NDIV = 1 + (IM - 1) / NTAB;
  const double AM = 1.0 / IM, EPS = 1.2e-7, RNMX = 1.0 - EPS;
  int32_t k;
  if (*idum <= 0 || *iy == 0) {
    *idum = std::max(-*idum, 1);
    for (int j = NTAB + 8; j >= 1; --j) {
      k = *idum / IQ;
      *idum = IA * (*idum - k * IQ) - IR * k;
      if (*idum < 0) *idum += IM;
      if (j <= NTAB) iv[j - 1] = *idum;
    }
    *iy = iv[0];
  }
  k = *idum / IQ;
  *idum = IA * (*idum - k * IQ) - IR * k;
  if (*idum < 0) *idum += IM;
  int32_t j = *iy / NDIV;  // Fortran j = 1 + iy/NDIV, 1-based
  *iy = iv[j];
  iv[j] = *idum;
  return std::min(AM * (double)(*iy), RNMX);
}

// Conditional periodic shift of a particle centre toward a point, the
// nearest-image idiom repeated throughout the reference, e.g.
// B/partlib.f90:981-982: if (c - p > nh) c -= n; if (c - p < -nh) c += n.
inline double near_img(double c, double p, int n, int nh) {
  if ((c - p) > (double)nh) c = c - (double)n;
  if ((c - p) < -(double)nh) c = c + (double)n;
  return c;
}

// Fortran x**2 is evaluated as x*x
inline double sq(double x) { return x * x; }

inline int wrap(int i, int n) {
  if (i < 0) return i + n;
  if (i >= n) return i - n;
  return i;
}

}  // namespace

struct Oracle {
  lbm_config cfg;
  int nx, ny, nz, nxh, nyh, nzh;
  int64_t N;
  bool channel;
  int npart = 0;
  bool particles_on = false;
  bool first_move = false;  // istep == irelease in beads_move
  int error = 0;
  std::string msg;

  // B/para.f90:91-175 derived constants
  double pi, pi2, tau, s1, s2, s4, s9, s10, s13, s16;
  double omegepsl, omegepslj, omegxx;
  double coef1, coef2, coef3, coef4, coef5, coef3i, coef4i;
  double val1, val2, val3, val4, val5, val6, val7, val8, val9;
  double val1i, val2i, val3i, val4i, val5i, val6i, val7i, val8i, val9i;
  double ww0, ww1, ww2, wwp[NPOP];
  double volp, amp, aip, tscale;

  std::vector<double> f, rho, ux, uy, uz, fx, fy, fz;
  std::vector<int32_t> ibnodes, isnodes, ibnodes0, isnodes0, ilink, mlink;
  std::vector<double> alink;

  std::vector<double> ypglb, ypglbp, wp, wpp, omgp, omgpp, dwdt, domgdt;
  std::vector<double> forcep, forcepp, torqp, torqpp, thetap, fHIp, flubp;
  std::vector<int32_t> ovlpflag;

  // forcing state, B/var_inc.f90:74-76 (6,5,5) Fortran order
  int32_t iseedf, iyf, ivf[32];
  double b1r[150], b2r[150], b3r[150], a1r[150], a2r[150], a3r[150];
  double kxr6[6], kyr5[5], kzr5[5];
  // particle RNG state (ranpp)
  int32_t iseedp, iyp, ivp[32];

  explicit Oracle(const lbm_config& c) : cfg(c) {
    nx = c.nx; ny = c.ny; nz = c.nz;
    nxh = nx / 2; nyh = ny / 2; nzh = nz / 2;
    N = (int64_t)nx * ny * nz;
    channel = (c.boundary == LBM_BC_XWALLS);
    para();
    f.assign(NPOP * N, 0.0);
    rho.assign(N, 0.0); ux.assign(N, 0.0); uy.assign(N, 0.0); uz.assign(N, 0.0);
    fx.assign(N, 0.0); fy.assign(N, 0.0); fz.assign(N, 0.0);
    ibnodes.assign(N, -1); isnodes.assign(N, -1);
    ibnodes0.assign(N, -1); isnodes0.assign(N, -1);
    int np = std::max(c.npart_max, 0);
    if (np > 0) {
      ilink.assign(18 * N, -1); mlink.assign(18 * N, -1); alink.assign(18 * N, 0.0);
    }
    auto v3 = [&](std::vector<double>& v) { v.assign(3 * (size_t)np, 0.0); };
    v3(ypglb); v3(ypglbp); v3(wp); v3(wpp); v3(omgp); v3(omgpp); v3(dwdt); v3(domgdt);
    v3(forcep); v3(forcepp); v3(torqp); v3(torqpp); v3(thetap); v3(fHIp); v3(flubp);
    ovlpflag.assign(np, 0);
    if (c.forcing == LBM_FORCING_CONSTANT) {
      std::fill(fy.begin(), fy.end(), c.force_y);
    }
  }

  // B/para.f90:1-288 (values that matter for the time step)
  void para() {
    pi = 4.0 * std::atan(1.0);
    pi2 = 2.0 * pi;
    tau = 3.0 * cfg.visc + 0.5;
    switch (cfg.mrt_type) {
      case 1: omegepsl = 0.0; omegepslj = -475.0 / 63.0; omegxx = 0.0; break;
      default: omegepsl = 3.0; omegepslj = -11.0 / 2.0; omegxx = -1.0 / 2.0; break;
    }
    s9 = 1.0 / tau;
    s13 = s9;
    switch (cfg.mrt_type) {
      case 1: s1 = 1.19; s2 = 1.4; s4 = 1.2; s10 = 1.4; s16 = 1.98; break;
      case 2: s1 = s9; s2 = s9; s4 = s9; s10 = s9; s16 = s9; break;
      default: s1 = 1.8; s2 = s1; s4 = s9; s10 = s1; s16 = s1; break;
    }
    coef1 = -2.0 / 3.0; coef2 = -11.0; coef3 = 8.0; coef4 = -4.0; coef5 = 2.0;
    coef3i = 1.0 / coef3; coef4i = 1.0 / coef4;
    val1 = 19.0; val2 = 2394.0; val3 = 252.0; val4 = 10.0; val5 = 40.0;
    val6 = 36.0; val7 = 72.0; val8 = 12.0; val9 = 24.0;
    val1i = 1.0 / val1; val2i = 1.0 / val2; val3i = 1.0 / val3; val4i = 1.0 / val4;
    val5i = 1.0 / val5; val6i = 1.0 / val6; val7i = 1.0 / val7; val8i = 1.0 / val8;
    val9i = 1.0 / val9;
    ww0 = 1.0 / 3.0; ww1 = 1.0 / 18.0; ww2 = 1.0 / 36.0;
    wwp[0] = 0.0;
    for (int ip = 1; ip <= 6; ++ip) wwp[ip] = ww1;   // para.f90:251-252
    for (int ip = 7; ip < NPOP; ++ip) wwp[ip] = ww2;
    volp = 4.0 / 3.0 * pi * (cfg.rad * cfg.rad * cfg.rad);      // para.f90:230-232
    amp = cfg.rhopart * volp;
    aip = 0.4 * amp * (cfg.rad * cfg.rad);
    tscale = pi2 * cfg.vscale / (double)ny;            // para.f90:60
    // forcing wavenumbers for the 6x5x5 low-mode block, para.f90:260-286
    // kxr(i) = int(i/2) for odd i and kxr(i+1) = kxr(i): 0, 0, 1, 1, 2, 2
    for (int i = 1; i <= 6; ++i) kxr6[i - 1] = (double)((i - 1) / 2);
    for (int j = 1; j <= 5; ++j) {
      int jj = (j > 3) ? j + ny - 5 : j;
      kyr5[j - 1] = (jj < ny / 2 + 2) ? (double)(jj - 1) : (double)(-(ny + 1 - jj));
      int kk = (j > 3) ? j + nz - 5 : j;
      kzr5[j - 1] = (kk < nz / 2 + 2) ? (double)(kk - 1) : (double)(-(nz + 1 - kk));
    }
    iseedf = -cfg.iseedf;  // para.f90:281-286
    std::memset(ivf, 0, sizeof(ivf));
    iyf = 0;
    for (int i = 0; i < 150; ++i) { b1r[i] = b2r[i] = b3r[i] = 0.0; a1r[i] = a2r[i] = a3r[i] = 0.0; }
    iseedp = cfg.iseedp;
    iyp = 0;
    std::memset(ivp, 0, sizeof(ivp));
  }

  inline int64_t nid(int i, int j, int k) const { return i + (int64_t)nx * (j + (int64_t)ny * k); }
  static inline int m655(int i, int j, int k) { return (i - 1) + 6 * (j - 1) + 30 * (k - 1); }

  // ---------------------------------------------------------------------------
  // FORCING, B/gaussian.f90:182-372 (box); C/collision.f90:335-347 (channel)
  void forcing() {
    if (cfg.forcing == LBM_FORCING_CONSTANT) {
      std::fill(fx.begin(), fx.end(), 0.0);
      std::fill(fy.begin(), fy.end(), cfg.force_y);
      std::fill(fz.begin(), fz.end(), 0.0);
      return;
    }
    if (cfg.forcing != LBM_FORCING_STOCHASTIC) return;
    double fr[150 * 3];
    const double smallx = 1.0e-18;
    const double xkf = std::sqrt(8.0);
    const double var = 447.31 * sq(cfg.vscale * tscale);
    const double tf = 0.038 / tscale;
    const double dt = 1.0;
    // white noise, gaussian.f90:201-215
    for (int mc = 1; mc <= 3; ++mc)
      for (int k = 1; k <= 5; ++k)
        for (int j = 1; j <= 5; ++j)
          for (int i = 1; i <= 6; i += 2) {
            int ip = i + 1;
            double cont1 = ran1(&iseedf, &iyf, ivf);
            if (cont1 < 1.e-6) cont1 = 1.e-6;
            double rmag = std::sqrt(-4.0 * var * dt * std::log(cont1) / tf);
            double rph = ran1(&iseedf, &iyf, ivf);
            fr[m655(i, j, k) + 150 * (mc - 1)] = rmag * std::cos(pi2 * rph);
            fr[m655(ip, j, k) + 150 * (mc - 1)] = rmag * std::sin(pi2 * rph);
          }
    // real-valued forcing in the k1 = 0 plane, gaussian.f90:220-236
    for (int mc = 1; mc <= 3; ++mc) {
      double* q = fr + 150 * (mc - 1);
      for (int k = 1; k <= 5; ++k) {
        int kk = 7 - k;
        if (k == 1) kk = 1;
        for (int j = 2; j <= 3; ++j) {
          int jj = 7 - j;
          q[m655(1, jj, kk)] = q[m655(1, j, k)];
          q[m655(2, jj, kk)] = -q[m655(2, j, k)];
        }
      }
      for (int k = 2; k <= 3; ++k) {
        int kk = 7 - k;
        q[m655(1, 1, kk)] = q[m655(1, 1, k)];
        q[m655(2, 1, kk)] = -q[m655(2, 1, k)];
      }
      q[m655(1, 1, 1)] = 0.0;
      q[m655(2, 1, 1)] = 0.0;
    }
    // OU update and solenoidal projection, gaussian.f90:243-274
    for (int k = 1; k <= 5; ++k)
      for (int j = 1; j <= 5; ++j)
        for (int i = 1; i <= 6; ++i) {
          int m = m655(i, j, k);
          double kx = kxr6[i - 1], ky = kyr5[j - 1], kz = kzr5[k - 1];
          double radm = std::sqrt(kx * kx + ky * ky + kz * kz);
          if (radm < xkf) {
            b1r[m] = b1r[m] * (1.0 - dt / tf) + fr[m];
            b2r[m] = b2r[m] * (1.0 - dt / tf) + fr[m + 150];
            b3r[m] = b3r[m] * (1.0 - dt / tf) + fr[m + 300];
            double t1 = kx * b1r[m], t2 = ky * b2r[m], t3 = kz * b3r[m];
            double divb = (t1 + t2 + t3) / sq(radm + smallx);
            if (radm == 0.0) divb = 0.0;
            a1r[m] = b1r[m] - kx * divb;
            a2r[m] = b2r[m] - ky * divb;
            a3r[m] = b3r[m] - kz * divb;
          } else {
            a1r[m] = 0.0; a2r[m] = 0.0; a3r[m] = 0.0;
          }
        }
    // gaussian.f90:277-307
    for (int i = 1; i <= 2; ++i) { a1r[m655(i, 1, 1)] = 0.0; a2r[m655(i, 1, 1)] = 0.0; a3r[m655(i, 1, 1)] = 0.0; }
    for (int k = 1; k <= 5; ++k) {
      int kk = 7 - k;
      if (k == 1) kk = 1;
      for (int j = 2; j <= 3; ++j) {
        int jj = 7 - j;
        a1r[m655(1, jj, kk)] = a1r[m655(1, j, k)]; a1r[m655(2, jj, kk)] = -a1r[m655(2, j, k)];
        a2r[m655(1, jj, kk)] = a2r[m655(1, j, k)]; a2r[m655(2, jj, kk)] = -a2r[m655(2, j, k)];
        a3r[m655(1, jj, kk)] = a3r[m655(1, j, k)]; a3r[m655(2, jj, kk)] = -a3r[m655(2, j, k)];
      }
    }
    for (int k = 2; k <= 3; ++k) {
      int kk = 7 - k;
      a1r[m655(1, 1, kk)] = a1r[m655(1, 1, k)]; a1r[m655(2, 1, kk)] = -a1r[m655(2, 1, k)];
      a2r[m655(1, 1, kk)] = a2r[m655(1, 1, k)]; a2r[m655(2, 1, kk)] = -a2r[m655(2, 1, k)];
      a3r[m655(1, 1, kk)] = a3r[m655(1, 1, k)]; a3r[m655(2, 1, kk)] = -a3r[m655(2, 1, k)];
    }
    synthesize(a1r, fx.data());
    synthesize(a2r, fy.data());
    synthesize(a3r, fz.data());
  }

  // Unnormalised inverse 3D transform of the low-mode block placed by
  // gaussian.f90:325-359 and transformed by mpifft3DCR (B/mpifft.f90:111-158):
  // complex backward transform over kz, then over ky, then the
  // complex-to-real transform over kx, each with exp(+2 pi i k n / N).
  // Only the 3x5x5 nonzero modes enter, so each stage is a direct sum over
  // them (the same arithmetic an FFT performs on a mostly-zero input).
  void synthesize(const double* a, double* out) const {
    const int NKX = 3, NK = 5;
    auto tw = [](int k, int n, int len, double* c, double* s) {
      int64_t m = ((int64_t)k * n) % len;
      if (m < 0) m += len;
      double ang = 2.0 * (4.0 * std::atan(1.0)) * (double)m / (double)len;
      *c = std::cos(ang); *s = std::sin(ang);
    };
    // stage 1: A(kx, ky, z)
    std::vector<double> Are(NKX * NK * nz), Aim(NKX * NK * nz);
    for (int kx = 0; kx < NKX; ++kx)
      for (int jy = 0; jy < NK; ++jy)
        for (int z = 0; z < nz; ++z) {
          double sr = 0.0, si = 0.0;
          for (int kz = 0; kz < NK; ++kz) {
            double cr = a[m655(2 * kx + 1, jy + 1, kz + 1)];
            double ci = a[m655(2 * kx + 2, jy + 1, kz + 1)];
            double c, s;
            tw((int)kzr5[kz], z, nz, &c, &s);
            sr += cr * c - ci * s;
            si += cr * s + ci * c;
          }
          Are[(kx * NK + jy) * nz + z] = sr;
          Aim[(kx * NK + jy) * nz + z] = si;
        }
    // stage 2 and 3
    std::vector<double> cx1(nx), sx1(nx), cx2(nx), sx2(nx);
    for (int x = 0; x < nx; ++x) { tw(1, x, nx, &cx1[x], &sx1[x]); tw(2, x, nx, &cx2[x], &sx2[x]); }
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y) {
        double Bre[NKX], Bim[NKX];
        for (int kx = 0; kx < NKX; ++kx) {
          double sr = 0.0, si = 0.0;
          for (int jy = 0; jy < NK; ++jy) {
            double ar = Are[(kx * NK + jy) * nz + z], ai = Aim[(kx * NK + jy) * nz + z];
            double c, s;
            tw((int)kyr5[jy], y, ny, &c, &s);
            sr += ar * c - ai * s;
            si += ar * s + ai * c;
          }
          Bre[kx] = sr; Bim[kx] = si;
        }
        for (int x = 0; x < nx; ++x) {
          double v = Bre[0] + 2.0 * (Bre[1] * cx1[x] - Bim[1] * sx1[x]) +
                     2.0 * (Bre[2] * cx2[x] - Bim[2] * sx2[x]);
          out[nid(x, y, z)] = v;
        }
      }
  }

  // ---------------------------------------------------------------------------
  // collision_MRT, B/collision.f90:8-210
  void collision_mrt() {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      if (ibnodes[n] >= 0) continue;
      double f9[NPOP], Fbar[NPOP];
      double rho9 = rho[n], ux9 = ux[n], uy9 = uy[n], uz9 = uz[n];
      double ux9s = ux9 * ux9, uy9s = uy9 * uy9, uz9s = uz9 * uz9;
      double fx9 = fx[n], fy9 = fy[n], fz9 = fz[n];
      double G3 = ux9 * fx9 + uy9 * fy9 + uz9 * fz9;
      Fbar[0] = -G3;
      for (int ip = 1; ip <= 6; ++ip) {
        double G1 = CIX[ip] * fx9 + CIY[ip] * fy9 + CIZ[ip] * fz9;
        double G2 = CIX[ip] * ux9 + CIY[ip] * uy9 + CIZ[ip] * uz9;
        Fbar[ip] = ww1 * (3. * G1 + 9. * G1 * G2 - 3. * G3);
      }
      for (int ip = 7; ip < NPOP; ++ip) {
        double G1 = CIX[ip] * fx9 + CIY[ip] * fy9 + CIZ[ip] * fz9;
        double G2 = CIX[ip] * ux9 + CIY[ip] * uy9 + CIZ[ip] * uz9;
        Fbar[ip] = ww2 * (3. * G1 + 9. * G1 * G2 - 3. * G3);
      }
      for (int ip = 0; ip < NPOP; ++ip) f9[ip] = f[ip * N + n] + Fbar[ip] / 2.;

      double t1 = ux9s + uy9s + uz9s;
      double eqm1 = -11.0 * rho9 + 19.0 * t1;
      double eqm2 = omegepsl * rho9 + omegepslj * t1;
      double eqm3 = coef1 * ux9, eqm4 = coef1 * uy9, eqm5 = coef1 * uz9;
      double eqm6 = 2.0 * ux9s - uy9s - uz9s;
      double eqm7 = omegxx * eqm6;
      double eqm8 = uy9s - uz9s;
      double eqm9 = omegxx * eqm8;
      double eqm10 = ux9 * uy9, eqm11 = uy9 * uz9, eqm12 = ux9 * uz9;
      double eqm13 = 0.0, eqm14 = 0.0, eqm15 = 0.0;

      double sum1 = f9[1] + f9[2] + f9[3] + f9[4] + f9[5] + f9[6];
      double sum2 = f9[7] + f9[8] + f9[9] + f9[10] + f9[11] + f9[12] + f9[13] + f9[14] +
                    f9[15] + f9[16] + f9[17] + f9[18];
      double sum3 = f9[7] - f9[8] + f9[9] - f9[10] + f9[11] - f9[12] + f9[13] - f9[14];
      double sum4 = f9[7] + f9[8] - f9[9] - f9[10] + f9[15] - f9[16] + f9[17] - f9[18];
      double sum5 = f9[11] + f9[12] - f9[13] - f9[14] + f9[15] + f9[16] - f9[17] - f9[18];
      double sum6 = f9[1] + f9[2];
      double sum7 = f9[3] + f9[4] + f9[5] + f9[6];
      double sum8 = f9[7] + f9[8] + f9[9] + f9[10] + f9[11] + f9[12] + f9[13] + f9[14];
      double sum9 = f9[15] + f9[16] + f9[17] + f9[18];
      double sum10 = f9[3] + f9[4] - f9[5] - f9[6];
      double sum11 = f9[7] + f9[8] + f9[9] + f9[10] - f9[11] - f9[12] - f9[13] - f9[14];

      double evlm1 = -30.0 * f9[0] + coef2 * sum1 + coef3 * sum2;
      double evlm2 = 12.0 * f9[0] + coef4 * sum1 + sum2;
      double evlm3 = coef4 * (f9[1] - f9[2]) + sum3;
      double evlm4 = coef4 * (f9[3] - f9[4]) + sum4;
      double evlm5 = coef4 * (f9[5] - f9[6]) + sum5;
      double evlm6 = coef5 * sum6 - sum7 + sum8 - coef5 * sum9;
      double evlm7 = coef4 * sum6 + coef5 * sum7 + sum8 - coef5 * sum9;
      double evlm8 = sum10 + sum11;
      double evlm9 = -coef5 * sum10 + sum11;
      double evlm10 = f9[7] - f9[8] - f9[9] + f9[10];
      double evlm11 = f9[15] - f9[16] - f9[17] + f9[18];
      double evlm12 = f9[11] - f9[12] - f9[13] + f9[14];
      double evlm13 = f9[7] - f9[8] + f9[9] - f9[10] - f9[11] + f9[12] - f9[13] + f9[14];
      double evlm14 = -f9[7] - f9[8] + f9[9] + f9[10] + f9[15] - f9[16] + f9[17] - f9[18];
      double evlm15 = f9[11] + f9[12] - f9[13] - f9[14] - f9[15] - f9[16] + f9[17] + f9[18];

      double eqmc1 = evlm1 - s1 * (evlm1 - eqm1);
      double eqmc2 = evlm2 - s2 * (evlm2 - eqm2);
      double eqmc3 = evlm3 - s4 * (evlm3 - eqm3);
      double eqmc4 = evlm4 - s4 * (evlm4 - eqm4);
      double eqmc5 = evlm5 - s4 * (evlm5 - eqm5);
      double eqmc6 = evlm6 - s9 * (evlm6 - eqm6);
      double eqmc7 = evlm7 - s10 * (evlm7 - eqm7);
      double eqmc8 = evlm8 - s9 * (evlm8 - eqm8);
      double eqmc9 = evlm9 - s10 * (evlm9 - eqm9);
      double eqmc10 = evlm10 - s13 * (evlm10 - eqm10);
      double eqmc11 = evlm11 - s13 * (evlm11 - eqm11);
      double eqmc12 = evlm12 - s13 * (evlm12 - eqm12);
      double eqmc13 = evlm13 - s16 * (evlm13 - eqm13);
      double eqmc14 = evlm14 - s16 * (evlm14 - eqm14);
      double eqmc15 = evlm15 - s16 * (evlm15 - eqm15);

      double tl1 = val1i * rho9;
      double tl2 = coef2 * val2i * eqmc1;
      double tl3 = coef3 * val2i * eqmc1;
      double tl4 = coef4 * val3i * eqmc2;
      double tl5 = val3i * eqmc2;
      double tl6 = val4i * ux9;
      double tl7 = val5i * eqmc3;
      double tl8 = val4i * uy9;
      double tl9 = val5i * eqmc4;
      double tl10 = val4i * uz9;
      double tl11 = val5i * eqmc5;
      double tl12 = val6i * eqmc6;
      double tl13 = val7i * eqmc7;
      double tl14 = val8i * eqmc8;
      double tl15 = val9i * eqmc9;
      double tl16 = -coef4i * eqmc10;
      double tl17 = -coef4i * eqmc11;
      double tl18 = -coef4i * eqmc12;
      double tl19 = coef3i * eqmc13;
      double tl20 = coef3i * eqmc14;
      double tl21 = coef3i * eqmc15;

      f9[0] = tl1 - 30.0 * val2i * eqmc1 + val8 * val3i * eqmc2;
      double suma = tl1 + tl2 + tl4;
      double sumb = tl1 + tl3 + tl5;
      double sumc = tl6 + coef4 * tl7;
      double sumd = coef5 * tl12 + coef4 * tl13;
      double sume = tl8 + coef4 * tl9;
      double sumf = -tl12 + coef5 * tl13 + tl14 - coef5 * tl15;
      double sumg = tl10 + coef4 * tl11;
      double sumh = -tl12 + coef5 * tl13 - tl14 + coef5 * tl15;
      double sumi = tl12 + tl13 + tl14 + tl15;
      double sumk = tl12 + tl13 - tl14 - tl15;
      double sump = -coef5 * tl12 - coef5 * tl13;
      double sum67 = tl6 + tl7, sum89 = tl8 + tl9, sum1011 = tl10 + tl11;

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

      for (int ip = 0; ip < NPOP; ++ip) f[ip * N + n] = f9[ip] + 0.5 * Fbar[ip];
    }
  }

  // rhoupdat, B/collision.f90:213-229
  void rhoupdat() {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      double r = f[n];
      for (int ip = 1; ip < NPOP; ++ip) r = r + f[ip * N + n];
      rho[n] = r;
    }
  }

  // macrovar, B/collision.f90:232-332 (channel: no x image, C/collision.f90:294-295)
  void macrovar() {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      double f9[NPOP];
      for (int ip = 0; ip < NPOP; ++ip) f9[ip] = f[ip * N + n];
      double sum1 = f9[7] - f9[10], sum2 = f9[9] - f9[8];
      double sum3 = f9[11] - f9[14], sum4 = f9[13] - f9[12];
      double sum5 = f9[15] - f9[18], sum6 = f9[17] - f9[16];
      double ux9 = f9[1] - f9[2] + sum1 + sum2 + sum3 + sum4;
      double uy9 = f9[3] - f9[4] + sum1 - sum2 + sum5 + sum6;
      double uz9 = f9[5] - f9[6] + sum3 - sum4 + sum5 - sum6;
      double rho9 = f9[0] + f9[1] + f9[2] + f9[3] + f9[4] + f9[5] + f9[6] + f9[7] + f9[8] +
                    f9[9] + f9[10] + f9[11] + f9[12] + f9[13] + f9[14] + f9[15] + f9[16] +
                    f9[17] + f9[18];
      ux[n] = ux9 + fx[n] / 2.;
      uy[n] = uy9 + fy[n] / 2.;
      uz[n] = uz9 + fz[n] / 2.;
      rho[n] = rho9;
    }
    if (!particles_on) return;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int64_t n = nid(i, j, k);
          if (ibnodes[n] <= 0) continue;
          int id = isnodes[n];
          double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5, zpnt = (double)(k + 1) - 0.5;
          double xc = ypglb[3 * id], yc = ypglb[3 * id + 1], zc = ypglb[3 * id + 2];
          if (!channel) xc = near_img(xc, xpnt, nx, nxh);
          yc = near_img(yc, ypnt, ny, nyh);
          zc = near_img(zc, zpnt, nz, nzh);
          double xx0 = xpnt - xc, yy0 = ypnt - yc, zz0 = zpnt - zc;
          double w1 = wp[3 * id], w2 = wp[3 * id + 1], w3 = wp[3 * id + 2];
          double o1 = omgp[3 * id], o2 = omgp[3 * id + 1], o3 = omgp[3 * id + 2];
          ux[n] = w1 + (o2 * zz0 - o3 * yy0);
          uy[n] = w2 + (o3 * xx0 - o1 * zz0);
          uz[n] = w3 + (o1 * yy0 - o2 * xx0);
          rho[n] = cfg.rhopart;
        }
  }

  // streaming, B/streaming.f90:2-171 (periodic push by c_i); channel
  // halfway bounce-back at x walls, C/streaming.f90:11-13,175-187
  void streaming() {
    std::vector<double> g(f.size());
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int64_t n = nid(i, j, k);
          g[n] = f[n];
          for (int ip = 1; ip < NPOP; ++ip) {
            int i2 = wrap(i + CIX[ip], nx), j2 = wrap(j + CIY[ip], ny), k2 = wrap(k + CIZ[ip], nz);
            g[ip * N + nid(i2, j2, k2)] = f[ip * N + n];
          }
        }
    if (channel) {
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
          int64_t nL = nid(0, j, k), nR = nid(nx - 1, j, k);
          for (int ip = 1; ip < NPOP; ++ip) {
            if (CIX[ip] == 1) g[ip * N + nL] = f[IPOPP[ip] * N + nL];
            if (CIX[ip] == -1) g[ip * N + nR] = f[IPOPP[ip] * N + nR];
          }
        }
    }
    f.swap(g);
  }

  // initpop, B/initial.f90:3-28 (rho' = 0, populations as deviations)
  void initpop() {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      double usqr = ux[n] * ux[n] + uy[n] * uy[n] + uz[n] * uz[n];
      usqr = 1.5 * usqr;
      rho[n] = 0.0;
      f[n] = ww0 * (rho[n] - usqr);
      for (int ip = 1; ip < NPOP; ++ip) {
        double G = CIX[ip] * ux[n] + CIY[ip] * uy[n] + CIZ[ip] * uz[n];
        double w = (ip <= 6) ? ww1 : ww2;
        f[ip * N + n] = w * (rho[n] + 3.0 * G + 4.5 * G * G - usqr);
      }
    }
  }

  // ---------------------------------------------------------------------------
  // ovlpchk, B/partlib.f90:118-171 (channel: no x image, C/partlib.f90:144-145)
  void ovlpchk(bool initial) {
    std::fill(ovlpflag.begin(), ovlpflag.end(), 0);
    for (int id = 0; id < npart - 1; ++id) {
      double xc = ypglb[3 * id], yc = ypglb[3 * id + 1], zc = ypglb[3 * id + 2];
      int iflag = 0;
      for (int ii = id + 1; ii < npart; ++ii) {
        double xb = ypglb[3 * ii], yb = ypglb[3 * ii + 1], zb = ypglb[3 * ii + 2];
        if (!channel) xb = near_img(xb, xc, nx, nxh);
        yb = near_img(yb, yc, ny, nyh);
        zb = near_img(zb, zc, nz, nzh);
        double dist = std::sqrt(sq(xc - xb) + sq(yc - yb) + sq(zc - zb));
        double hgap = dist - 2.0 * cfg.rad;
        if (initial) hgap = hgap - cfg.mingap;
        if (hgap < 0.0) { iflag = 1; break; }
      }
      if (iflag > 0) ovlpflag[id] = 1;
    }
  }

  // initpartpos, B/partlib.f90:1-80 (channel x range C/partlib.f90:10-24)
  int initpartpos(int np) {
    npart = np;
    iseedp = -cfg.iseedp;
    iyp = 0;
    std::memset(ivp, 0, sizeof(ivp));
    std::vector<int32_t> flagt(np, 1);
    const double radpgap = cfg.rad + cfg.mingap_w;
    for (int iter = 0; iter < 100000; ++iter) {
      for (int ip = 0; ip < np; ++ip) {
        if (flagt[ip] > 0) {
          if (channel)
            ypglb[3 * ip] = radpgap + ((double)nx - 2.0 * radpgap) * ran1(&iseedp, &iyp, ivp);
          else
            ypglb[3 * ip] = (double)nx * ran1(&iseedp, &iyp, ivp);
          ypglb[3 * ip + 1] = (double)ny * ran1(&iseedp, &iyp, ivp);
          ypglb[3 * ip + 2] = (double)nz * ran1(&iseedp, &iyp, ivp);
        }
      }
      ovlpchk(true);
      int cnt = 0;
      for (int ip = 0; ip < np; ++ip) { flagt[ip] = ovlpflag[ip]; cnt += (ovlpflag[ip] != 0); }
      if (cnt == 0) return 0;
    }
    return LBM_ERR_OVERLAP;
  }

  // initpartvel, B/partlib.f90:177-263 with trilinear (iflag = 1),
  // B/partlib.f90:320-831 (channel: C/partlib.f90:182-268, 325-836, the same
  // but with the x wrap of 356-358 commented out).  One process holds the
  // whole domain, so the halo planes exchng1 brings in (tmpL = plane nz,
  // tmpR = plane 1, tmpU = row 1, tmpD = row ny, with their corners) are the
  // periodic images, and every case of trilinear reads u at the nodes
  // (i|ip1, j|jp1, k|kp1) wrapped into 1..n.  Node i (1-based) sits at
  // i - 0.5.  The weights and the sum are formed in the reference's order.
  // Returns the 0-based index of the first centre whose cell leaves the grid
  // (x + 0.5 outside [0, n + 1) along an open axis, outside [1, nx) along a
  // channel's walls: the reference reads outside its arrays there), else -1.
  int initpartvel(int np) {
    const double* uv[3] = {ux.data(), uy.data(), uz.data()};
    for (int ip = 0; ip < np; ++ip) {
      const double xc = ypglb[3 * ip], yc = ypglb[3 * ip + 1], zc = ypglb[3 * ip + 2];
      const double sx = (xc + 0.5) / 1.0, sy = (yc - 0.0 + 0.5) / 1.0, sz = (zc - 0.0 + 0.5) / 1.0;
      if (!((channel ? (sx >= 1.0 && sx < nx) : (sx >= 0.0 && sx < nx + 1.0)) && sy >= 0.0 &&
            sy < ny + 1.0 && sz >= 0.0 && sz < nz + 1.0))
        return ip;
      int i = (int)((xc + 0.5) / 1.0);
      int j = (int)((yc - 0.0 + 0.5) / 1.0);
      int k = (int)((zc - 0.0 + 0.5) / 1.0);
      int ip1 = i + 1, jp1 = j + 1, kp1 = k + 1;
      const double tx = (xc + 0.5 - (double)i) / 1.0;
      const double ty = (yc - 0.0 + 0.5 - (double)j) / 1.0;
      const double tz = (zc - 0.0 + 0.5 - (double)k) / 1.0;
      const double tx0 = 1.0 - tx, ty0 = 1.0 - ty, tz0 = 1.0 - tz;
      if (!channel) {
        if (i == 0) i = nx;
        if (ip1 > nx) ip1 = 1;
      }
      if (j == 0) j = ny;
      if (jp1 > ny) jp1 = 1;
      if (k == 0) k = nz;
      if (kp1 > nz) kp1 = 1;
      auto at = [&](const double* u, int a, int b, int c) {
        return u[((int64_t)(c - 1) * ny + (b - 1)) * nx + (a - 1)];
      };
      for (int d = 0; d < 3; ++d) {
        const double* u = uv[d];
        const double v1 = at(u, i, j, k), v2 = at(u, ip1, j, k), v3 = at(u, ip1, jp1, k),
                     v4 = at(u, i, jp1, k), v5 = at(u, i, j, kp1), v6 = at(u, ip1, j, kp1),
                     v7 = at(u, ip1, jp1, kp1), v8 = at(u, i, jp1, kp1);
        wp[3 * ip + d] = tx0 * ty0 * tz0 * v1 + tx * ty0 * tz0 * v2 + tx * ty * tz0 * v3 +
                         tx0 * ty * tz0 * v4 + tx0 * ty0 * tz * v5 + tx * ty0 * tz * v6 +
                         tx * ty * tz * v7 + tx0 * ty * tz * v8;
      }
    }
    return -1;
  }

  // Release particles at given positions and velocities: the irelease block
  // of B/main.f90:149-165 with initpartvel/initpartomg replaced by inputs.
  void release(int np) {
    npart = np;
    particles_on = true;
    first_move = true;
    std::copy(ypglb.begin(), ypglb.end(), ypglbp.begin());
    beads_links();
  }

  // restart with particles (B/main.f90:129-132): the state vectors were set
  // from a checkpoint; rebuild the flags and links, the next move is not the
  // first after release
  void restore(int np) {
    npart = np;
    particles_on = np > 0;
    first_move = false;
    if (np > 0) beads_links();
  }

  // beads_links, B/partlib.f90:934-1058 (channel: C/partlib.f90:939-1058)
  void beads_links() {
    std::fill(ilink.begin(), ilink.end(), -1);
    std::fill(mlink.begin(), mlink.end(), -1);
    std::fill(ibnodes.begin(), ibnodes.end(), -1);
    std::fill(isnodes.begin(), isnodes.end(), -1);
    std::fill(alink.begin(), alink.end(), 0.0);
    const double rad = cfg.rad;
    const double radp2 = rad * 1.0 + 2.0;
    for (int ip = 0; ip < npart; ++ip) {
      // xc, yc, zc keep their shifted values across loop iterations, as in
      // the reference (they are never reset inside the loop nest)
      double xc = ypglb[3 * ip], yc = ypglb[3 * ip + 1], zc = ypglb[3 * ip + 2];
      for (int k = 1; k <= nz; ++k) {
        double zpnt = (double)k - 0.5 + 0.0;
        zc = near_img(zc, zpnt, nz, nzh);
        double zz0 = zpnt - zc;
        if (!(std::fabs(zz0) <= radp2)) continue;
        for (int j = 1; j <= ny; ++j) {
          double ypnt = (double)j - 0.5 + 0.0;
          yc = near_img(yc, ypnt, ny, nyh);
          double yy0 = ypnt - yc;
          if (channel) {
            if (!(std::sqrt(yy0 * yy0 + zz0 * zz0) <= radp2)) continue;
          } else {
            if (!(std::fabs(yy0) <= radp2)) continue;
          }
          for (int i = 1; i <= nx; ++i) {
            double xpnt = (double)i - 0.5;
            double xx0, rr0;
            if (channel) {
              xx0 = xpnt - xc;
              rr0 = sq(xx0) + sq(yy0) + sq(zz0);
              if (!(std::sqrt(rr0) <= radp2)) continue;
            } else {
              xc = near_img(xc, xpnt, nx, nxh);
              xx0 = xpnt - xc;
              if (!(std::fabs(xx0) <= radp2)) continue;
              rr0 = sq(xx0) + sq(yy0) + sq(zz0);
            }
            double rr01 = rr0 - sq(rad * 1.0);
            int64_t n = nid(i - 1, j - 1, k - 1);
            if (rr01 <= 0.0) {
              ibnodes[n] = 1;
              isnodes[n] = ip;
            } else {
              for (int ipop = 1; ipop < NPOP; ++ipop) {
                int imove = i + CIX[ipop], jmove = j + CIY[ipop], kmove = k + CIZ[ipop];
                double xx1 = (double)imove - 0.5 - xc;
                double yy1 = (double)jmove - 0.5 - yc + 0.0;
                double zz1 = (double)kmove - 0.5 - zc + 0.0;
                double rr1 = sq(xx1) + sq(yy1) + sq(zz1);
                double rr11 = rr1 - sq(rad * 1.0);
                if (rr11 <= 0.0) {
                  int64_t l = (int64_t)(ipop - 1) * N + n;
                  ilink[l] = 1;
                  mlink[l] = ip;
                  double aa = rr0 + rr1 - 2.0 * (xx0 * xx1 + yy0 * yy1 + zz0 * zz1);
                  double bb = xx1 * (xx0 - xx1) + yy1 * (yy0 - yy1) + zz1 * (zz0 - zz1);
                  double cc = rr11;
                  double alpha0 = bb / aa;
                  double alpha1 = std::sqrt(sq(alpha0) - cc / aa);
                  double alpha = -alpha0 + alpha1;
                  alpha = 1.0 - alpha;
                  alink[l] = alpha;
                  if (alpha < 0.0 || alpha > 1.0) {
                    if (!error) { error = LBM_ERR_ALPHA; msg = "link fraction outside [0,1]"; }
                  }
                }
              }
            }
          }
        }
      }
    }
  }

  // beads_collision, B/partlib.f90:1363-1703 (channel wall cases
  // C/partlib.f90:1458-1462,1483-1487,1532-1537): interpolated bounce-back
  // on moving spheres plus momentum-exchange force and torque.
  void beads_collision() {
    std::vector<double> fHIp0(3 * (size_t)npart, 0.0), torqp0(3 * (size_t)npart, 0.0);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int64_t n = nid(i, j, k);
          for (int ipop = 1; ipop < NPOP; ++ipop) {
            int64_t l = (int64_t)(ipop - 1) * N + n;
            if (!(ilink[l] > 0)) continue;
            int id = mlink[l];
            double alpha = alink[l];
            int ipp = IPOPP[ipop];
            double xc = ypglb[3 * id], yc = ypglb[3 * id + 1], zc = ypglb[3 * id + 2];
            double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5, zpnt = (double)(k + 1) - 0.5;
            if (!channel) xc = near_img(xc, xpnt, nx, nxh);
            yc = near_img(yc, ypnt, ny, nyh);
            zc = near_img(zc, zpnt, nz, nzh);
            double w1 = wp[3 * id], w2 = wp[3 * id + 1], w3 = wp[3 * id + 2];
            double omg1 = omgp[3 * id], omg2 = omgp[3 * id + 1], omg3 = omgp[3 * id + 2];
            int ix = CIX[ipop], iy = CIY[ipop], iz = CIZ[ipop];
            int im1 = i - ix, jm1 = wrap(j - iy, ny), km1 = wrap(k - iz, nz);
            int im2 = i - 2 * ix, jm2 = wrap(j - 2 * iy, ny), km2 = wrap(k - 2 * iz, nz);
            int ip1 = i + ix, jp1 = wrap(j + iy, ny), kp1 = wrap(k + iz, nz);
            bool out1 = false, out2 = false, outp = false;
            if (channel) {
              out1 = (im1 < 0 || im1 >= nx);
              out2 = (im2 < 0 || im2 >= nx);
              outp = (ip1 < 0 || ip1 >= nx);
            } else {
              if (im1 < 0) im1 += nx; if (im1 >= nx) im1 -= nx;
              if (im2 < 0) im2 += nx; if (im2 >= nx) im2 -= nx;
              if (ip1 < 0) ip1 += nx; if (ip1 >= nx) ip1 -= nx;
            }
            double xx0 = xpnt + (double)ix * alpha - xc;
            double yy0 = ypnt + (double)iy * alpha - yc;
            double zz0 = zpnt + (double)iz * alpha - zc;
            double ff1 = f[ipop * N + n];
            double uwx = w1 + omg2 * zz0 - omg3 * yy0;
            double uwy = w2 + omg3 * xx0 - omg1 * zz0;
            double uwz = w3 + omg1 * yy0 - omg2 * xx0;
            double uwpro = uwx * (double)ix + uwy * (double)iy + uwz * (double)iz;
            double f9, ff2, ff3;
            int ibm1, ibm2;
            if (alpha <= 0.5) {
              if (out1) { ibm1 = 2; ff2 = 0.0; }
              else { int64_t m1 = nid(im1, jm1, km1); ff2 = f[ipop * N + m1]; ibm1 = ibnodes[m1]; }
              if (out2) { ibm2 = 2; ff3 = 0.0; }
              else { int64_t m2 = nid(im2, jm2, km2); ff3 = f[ipop * N + m2]; ibm2 = ibnodes[m2]; }
              if (ibm1 > 0) {
                f9 = ff1 - 6.0 * wwp[ipop] * uwpro;
              } else if (ibm2 > 0) {
                f9 = 2.0 * alpha * (ff1 - ff2) + ff2 - 6.0 * wwp[ipop] * uwpro;
              } else {
                double c1 = alpha * (1.0 + 2.0 * alpha);
                double c2 = 1.0 - 4.0 * alpha * alpha;
                double c3 = -alpha * (1.0 - 2.0 * alpha);
                f9 = c1 * ff1 + c2 * ff2 + c3 * ff3 - 6.0 * wwp[ipop] * uwpro;
              }
            } else {
              ff2 = f[ipp * N + n];
              if (out1) { ibm1 = 2; ff3 = 0.0; }
              else { int64_t m1 = nid(im1, jm1, km1); ff3 = f[ipp * N + m1]; ibm1 = ibnodes[m1]; }
              if (ibm1 > 0) {
                double c1 = 0.5 / alpha;
                double c2 = 1.0 - c1;
                f9 = c1 * ff1 + c2 * ff2 - 6.0 * wwp[ipop] * c1 * uwpro;
              } else {
                double c1 = 1.0 / alpha / (2.0 * alpha + 1.0);
                double c2 = (2.0 * alpha - 1.0) / alpha;
                double c3 = 1.0 - c1 - c2;
                f9 = c1 * ff1 + c2 * ff2 + c3 * ff3 - 6.0 * wwp[ipop] * c1 * uwpro;
              }
            }
            // the reference writes f(ipp, ip1, jp1, kp1) even when ip1 lies
            // beyond a channel wall (out of bounds); here that store is dropped
            if (!outp) f[ipp * N + nid(ip1, jp1, kp1)] = f9;
            double dff = ff1 + f9;
            double dxmom = dff * (double)ix, dymom = dff * (double)iy, dzmom = dff * (double)iz;
            fHIp0[3 * id] = fHIp0[3 * id] + dxmom;
            fHIp0[3 * id + 1] = fHIp0[3 * id + 1] + dymom;
            fHIp0[3 * id + 2] = fHIp0[3 * id + 2] + dzmom;
            torqp0[3 * id] = torqp0[3 * id] + dzmom * yy0 - dymom * zz0;
            torqp0[3 * id + 1] = torqp0[3 * id + 1] + dxmom * zz0 - dzmom * xx0;
            torqp0[3 * id + 2] = torqp0[3 * id + 2] + dymom * xx0 - dxmom * yy0;
          }
        }
    std::copy(fHIp0.begin(), fHIp0.end(), fHIp.begin());
    std::copy(torqp0.begin(), torqp0.end(), torqp.begin());
  }

  // beads_lubforce, B/partlib.f90:2211-2292; channel C/partlib.f90:2245-2369
  void beads_lubforce() {
    const double rad = cfg.rad, mingap = cfg.mingap;
    double dist0 = 2.0 * rad + mingap;
    std::vector<double> fl(3 * (size_t)npart, 0.0);
    const double fpc = cfg.fpc;
    for (int id = 0; id < npart - 1; ++id) {
      double xc = ypglb[3 * id], yc = ypglb[3 * id + 1], zc = ypglb[3 * id + 2];
      for (int jj = id + 1; jj < npart; ++jj) {
        double xb = ypglb[3 * jj], yb = ypglb[3 * jj + 1], zb = ypglb[3 * jj + 2];
        if (!channel) xb = near_img(xb, xc, nx, nxh);
        yb = near_img(yb, yc, ny, nyh);
        zb = near_img(zb, zc, nz, nzh);
        double dxij = xc - xb, dyij = yc - yb, dzij = zc - zb;
        double dist = std::sqrt(dxij * dxij + dyij * dyij + dzij * dzij);
        double hgap = dist - 2.0 * rad;
        if (channel) {
          if (dist < dist0) {
            double dist1 = 0.0;
            if (hgap < 0.0) dist1 = -hgap;
            double fp = (sq((dist0 - dist) / mingap) / cfg.stf0 + dist1 / mingap / cfg.stf1) * fpc;
            double fpd = fp / dist;
            fl[3 * id] = fl[3 * id] + fpd * dxij;
            fl[3 * id + 1] = fl[3 * id + 1] + fpd * dyij;
            fl[3 * id + 2] = fl[3 * id + 2] + fpd * dzij;
            fl[3 * jj] = fl[3 * jj] - fpd * dxij;
            fl[3 * jj + 1] = fl[3 * jj + 1] - fpd * dyij;
            fl[3 * jj + 2] = fl[3 * jj + 2] - fpd * dzij;
          }
        } else {
          double fp = 0.0;
          if (dist < dist0) {
            double dist1 = 0.0;
            if (hgap < 0.0) dist1 = -hgap;
            fp = (sq((dist0 - dist) / mingap) / cfg.stf0 + dist1 / mingap / cfg.stf1) * fpc;
          }
          double fpd = fp / dist;
          fl[3 * id] = fl[3 * id] + fpd * dxij;
          fl[3 * id + 1] = fl[3 * id + 1] + fpd * dyij;
          fl[3 * id + 2] = fl[3 * id + 2] + fpd * dzij;
          fl[3 * jj] = fl[3 * jj] - fpd * dxij;
          fl[3 * jj + 1] = fl[3 * jj + 1] - fpd * dyij;
          fl[3 * jj + 2] = fl[3 * jj + 2] - fpd * dzij;
        }
      }
    }
    if (channel) {
      // particle-wall lubrication, C/partlib.f90:2316-2355
      const double mw = cfg.mingap_w;
      double d0 = mw + rad;
      for (int id = 0; id < npart; ++id) {
        double xd = ypglb[3 * id];
        double dist = xd, hgap = dist - rad;
        if (dist < d0) {
          double dist1 = 0.0;
          if (hgap < 0.0) dist1 = -hgap;
          double fp = (sq((d0 - dist) / mw) / cfg.stf0_w + dist1 / mw / cfg.stf1_w) * fpc;
          fl[3 * id] = fl[3 * id] + fp;
        }
        dist = (double)nx - xd;
        hgap = dist - rad;
        if (dist < d0) {
          double dist1 = 0.0;
          if (hgap < 0.0) dist1 = -hgap;
          double fp = (sq((d0 - dist) / mw) / cfg.stf0_w + dist1 / mw / cfg.stf1_w) * fpc;
          fl[3 * id] = fl[3 * id] - fp;
        }
      }
    }
    std::copy(fl.begin(), fl.end(), flubp.begin());
  }

  // beads_move, B/partlib.f90:2295-2394 (gravity/pressure term 2332 / C 2409)
  void beads_move() {
    const double dt = 1.0;
    if (first_move) std::fill(thetap.begin(), thetap.end(), 0.0);
    wpp = wp;
    omgpp = omgp;
    for (int id = 0; id < npart; ++id) {
      double* fp = &forcep[3 * id];
      double* fpp = &forcepp[3 * id];
      double dwdtn[3], domgdtn[3];
      for (int c = 0; c < 3; ++c) fp[c] = fHIp[3 * id + c] + flubp[3 * id + c];
      fp[1] = fp[1] + cfg.body_force_y;
      if (first_move) for (int c = 0; c < 3; ++c) fpp[c] = fp[c];
      for (int c = 0; c < 3; ++c) dwdtn[c] = 0.5 * (fp[c] + fpp[c]) / amp;
      if (first_move) for (int c = 0; c < 3; ++c) dwdt[3 * id + c] = dwdtn[c];
      for (int c = 0; c < 3; ++c) wp[3 * id + c] = wpp[3 * id + c] + 0.5 * dt * (dwdt[3 * id + c] + dwdtn[c]);
      for (int c = 0; c < 3; ++c) ypglb[3 * id + c] = ypglb[3 * id + c] + 0.5 * dt * (wp[3 * id + c] + wpp[3 * id + c]);
      if (first_move) for (int c = 0; c < 3; ++c) torqpp[3 * id + c] = torqp[3 * id + c];
      for (int c = 0; c < 3; ++c) domgdtn[c] = 0.5 * (torqp[3 * id + c] + torqpp[3 * id + c]) / aip;
      if (first_move) for (int c = 0; c < 3; ++c) domgdt[3 * id + c] = domgdtn[c];
      for (int c = 0; c < 3; ++c) omgp[3 * id + c] = omgpp[3 * id + c] + 0.5 * dt * (domgdt[3 * id + c] + domgdtn[c]);
      for (int c = 0; c < 3; ++c) thetap[3 * id + c] = thetap[3 * id + c] + 0.5 * dt * (omgp[3 * id + c] + omgpp[3 * id + c]);
      for (int c = 0; c < 3; ++c) {
        dwdt[3 * id + c] = dwdtn[c];
        domgdt[3 * id + c] = domgdtn[c];
        fpp[c] = fp[c];
        torqpp[3 * id + c] = torqp[3 * id + c];
      }
    }
    first_move = false;
    ibnodes0 = ibnodes;
    isnodes0 = isnodes;
  }

  // beads_redistribute on one domain: periodic wrap (B/partlib.f90:2600-2613;
  // channel wraps y and z only, C/partlib.f90:2678-2699), ypglbp save (2624)
  // and the overlap check that aborts the reference (2630-2646).
  int beads_redistribute() {
    std::vector<double> old = ypglb;
    for (int id = 0; id < npart; ++id) {
      double xc = ypglb[3 * id], yc = ypglb[3 * id + 1], zc = ypglb[3 * id + 2];
      if (!channel) {
        if (xc >= (double)nx) ypglb[3 * id] = ypglb[3 * id] - (double)nx;
        if (xc < 0.0) ypglb[3 * id] = ypglb[3 * id] + (double)nx;
      }
      if (yc >= (double)ny) ypglb[3 * id + 1] = ypglb[3 * id + 1] - (double)ny;
      if (yc < 0.0) ypglb[3 * id + 1] = ypglb[3 * id + 1] + (double)ny;
      if (zc >= (double)nz) ypglb[3 * id + 2] = ypglb[3 * id + 2] - (double)nz;
      if (zc < 0.0) ypglb[3 * id + 2] = ypglb[3 * id + 2] + (double)nz;
    }
    ypglbp = ypglb_prev;
    ovlpchk(false);
    for (int id = 0; id < npart; ++id)
      if (ovlpflag[id]) { error = LBM_ERR_OVERLAP; msg = "particles overlap after move"; return error; }
    return 0;
  }
  std::vector<double> ypglb_prev;  // ypglb before beads_move of this step

  // feqpnt, B/partlib.f90:3222-3247
  void feqpnt(double u9, double v9, double w9, double rho9, double* feq9) const {
    double usqr = u9 * u9 + v9 * v9 + w9 * w9;
    usqr = 1.5 * usqr;
    feq9[0] = ww0 * (rho9 - usqr);
    for (int ip = 1; ip <= 6; ++ip) {
      double G = CIX[ip] * u9 + CIY[ip] * v9 + CIZ[ip] * w9;
      feq9[ip] = ww1 * (rho9 + 3.0 * G + 4.5 * G * G - usqr);
    }
    for (int ip = 7; ip < NPOP; ++ip) {
      double G = CIX[ip] * u9 + CIY[ip] * v9 + CIZ[ip] * w9;
      feq9[ip] = ww2 * (rho9 + 3.0 * G + 4.5 * G * G - usqr);
    }
  }

  // beads_filling, B/partlib.f90:2846-3094 (channel walls C/partlib.f90:3026-3035,
  // 3108-3114; channel fallback density 0, C/partlib.f90:3165)
  void beads_filling() {
    const double rad = cfg.rad;
    const double sq2 = std::sqrt(2.0);
    // neighbour query: returns false when the neighbour lies beyond a wall
    auto nb = [&](int i, int j, int k, int ip, int64_t* m) -> bool {
      int i2 = i + CIX[ip], j2 = wrap(j + CIY[ip], ny), k2 = wrap(k + CIZ[ip], nz);
      if (channel) { if (i2 < 0 || i2 >= nx) return false; }
      else i2 = wrap(i2, nx);
      *m = nid(i2, j2, k2);
      return true;
    };
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int64_t n = nid(i, j, k);
          if (!(ibnodes0[n] > 0 && ibnodes[n] < 0)) continue;
          int id = isnodes0[n];
          double xc = ypglbp[3 * id] * 1.0, yc = ypglbp[3 * id + 1] * 1.0, zc = ypglbp[3 * id + 2] * 1.0;
          double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5 + 0.0, zpnt = (double)(k + 1) - 0.5 + 0.0;
          if (!channel) xc = near_img(xc, xpnt, nx, nxh);
          yc = near_img(yc, ypnt, ny, nyh);
          zc = near_img(zc, zpnt, nz, nzh);
          double w1 = -0.5 * (wp[3 * id] * 1.0 + wpp[3 * id] * 1.0);
          double w2 = -0.5 * (wp[3 * id + 1] * 1.0 + wpp[3 * id + 1] * 1.0);
          double w3 = -0.5 * (wp[3 * id + 2] * 1.0 + wpp[3 * id + 2] * 1.0);
          double omg1 = -0.5 * (omgp[3 * id] * 1.0 + omgpp[3 * id] * 1.0);
          double omg2 = -0.5 * (omgp[3 * id + 1] * 1.0 + omgpp[3 * id + 1] * 1.0);
          double omg3 = -0.5 * (omgp[3 * id + 2] * 1.0 + omgpp[3 * id + 2] * 1.0);
          double aa = w1 * w1 + w2 * w2 + w3 * w3;
          double bb = (xpnt - xc) * w1 + (ypnt - yc) * w2 + (zpnt - zc) * w3;
          double cc = sq(xpnt - xc) + sq(ypnt - yc) + sq(zpnt - zc) - sq(rad * 1.0);
          double ddt0 = bb / aa;
          double ddt1 = std::sqrt(sq(ddt0) - cc / aa);
          double ddt = -ddt0 + ddt1;
          if (ddt < 0.0) ddt = 0.0;
          if (ddt > 1.0) ddt = 1.0;
          double xp1 = xpnt + w1 * ddt, yp1 = ypnt + w2 * ddt, zp1 = zpnt + w3 * ddt;
          double xp2 = xp1 + (omg2 * (zp1 - zc) - omg3 * (yp1 - yc)) * ddt;
          double yp2 = yp1 + (omg3 * (xp1 - xc) - omg1 * (zp1 - zc)) * ddt;
          double zp2 = zp1 + (omg1 * (yp1 - yc) - omg2 * (xp1 - xc)) * ddt;
          double xx0 = xp2 - xc, yy0 = yp2 - yc, zz0 = zp2 - zc;
          double prod0 = -100.0;
          int ipmx = 0;  // the reference leaves ipmx undefined if no prod > -100
          for (int ipop = 1; ipop < NPOP; ++ipop) {
            double prod = (double)CIX[ipop] * xx0 + (double)CIY[ipop] * yy0 + (double)CIZ[ipop] * zz0;
            if (ipop <= 6) prod = prod * sq2;
            if (prod > prod0) { ipmx = ipop; prod0 = prod; }
          }
          double f9[NPOP], feq9[NPOP];
          int64_t m;
          bool ok = (ipmx > 0) && nb(i, j, k, ipmx, &m);
          if (ok && ibnodes[m] < 0 && ibnodes0[m] < 0) {
            double rho9 = 0.0, u9 = 0.0, v9 = 0.0, w9 = 0.0;
            for (int ip = 0; ip < NPOP; ++ip) f9[ip] = f[ip * N + m];
            for (int ip = 0; ip < NPOP; ++ip) {
              rho9 = rho9 + f9[ip];
              u9 = u9 + (double)CIX[ip] * f9[ip];
              v9 = v9 + (double)CIY[ip] * f9[ip];
              w9 = w9 + (double)CIZ[ip] * f9[ip];
            }
            feqpnt(u9, v9, w9, rho9, feq9);
            for (int ip = 0; ip < NPOP; ++ip) f[ip * N + n] = f9[ip] - feq9[ip];
          } else {
            for (int ip = 0; ip < NPOP; ++ip) f[ip * N + n] = 0.0;
          }
          int nghb = 0;
          double rho9 = 0.0;
          for (int ipop = 1; ipop < NPOP; ++ipop) {
            if (!nb(i, j, k, ipop, &m)) continue;
            if (ibnodes[m] < 0 && ibnodes0[m] < 0) {
              nghb = nghb + 1;
              for (int ii = 0; ii < NPOP; ++ii) rho9 = rho9 + f[ii * N + m];
            }
          }
          if (nghb > 0) rho9 = rho9 / (double)nghb;
          else rho9 = channel ? 0.0 : cfg.rho0;
          xx0 = xpnt - xc; yy0 = ypnt - yc; zz0 = zpnt - zc;
          w1 = wp[3 * id]; w2 = wp[3 * id + 1]; w3 = wp[3 * id + 2];
          omg1 = omgp[3 * id]; omg2 = omgp[3 * id + 1]; omg3 = omgp[3 * id + 2];
          double u9 = w1 + omg2 * zz0 - omg3 * yy0;
          double v9 = w2 + omg3 * xx0 - omg1 * zz0;
          double w9 = w3 + omg1 * yy0 - omg2 * xx0;
          feqpnt(u9, v9, w9, rho9, feq9);
          for (int ip = 0; ip < NPOP; ++ip) f[ip * N + n] = f[ip * N + n] + feq9[ip];
        }
  }

  // one pass of the main loop, B/main.f90:172-188
  int step() {
    forcing();
    collision_mrt();
    if (particles_on) beads_collision();
    streaming();
    if (particles_on) {
      beads_lubforce();
      ypglb_prev = ypglb;
      beads_move();
      if (beads_redistribute() != 0) return error;
      beads_links();
      beads_filling();
    }
    macrovar();
    return error;
  }
};

// ----------------------------------------------------------------------------
// C interface used by the Python test harness (ctypes)
extern "C" {

void* orc_create(const lbm_config* cfg) { return new Oracle(*cfg); }
void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

// Raw pointer to a named state array; sizes follow the layout notes above.
void* orc_field(void* h, const char* name) {
  Oracle* o = static_cast<Oracle*>(h);
  std::string s(name);
#define F(x) if (s == #x) return (void*)o->x.data();
  F(f) F(rho) F(ux) F(uy) F(uz) F(fx) F(fy) F(fz)
  F(ibnodes) F(isnodes) F(ibnodes0) F(isnodes0) F(ilink) F(mlink) F(alink)
  F(ypglb) F(ypglbp) F(wp) F(wpp) F(omgp) F(omgpp) F(dwdt) F(domgdt)
  F(forcep) F(forcepp) F(torqp) F(torqpp) F(thetap) F(fHIp) F(flubp)
#undef F
  if (s == "b1r") return o->b1r;
  if (s == "b2r") return o->b2r;
  if (s == "b3r") return o->b3r;
  if (s == "a1r") return o->a1r;
  if (s == "a2r") return o->a2r;
  if (s == "a3r") return o->a3r;
  if (s == "ivf") return o->ivf;
  if (s == "iseedf") return &o->iseedf;
  if (s == "iyf") return &o->iyf;
  return nullptr;
}

int orc_error(void* h) { return static_cast<Oracle*>(h)->error; }
int orc_npart(void* h) { return static_cast<Oracle*>(h)->npart; }

void orc_forcing(void* h) { static_cast<Oracle*>(h)->forcing(); }
void orc_collision_mrt(void* h) { static_cast<Oracle*>(h)->collision_mrt(); }
void orc_beads_collision(void* h) { static_cast<Oracle*>(h)->beads_collision(); }
void orc_streaming(void* h) { static_cast<Oracle*>(h)->streaming(); }
void orc_beads_lubforce(void* h) { static_cast<Oracle*>(h)->beads_lubforce(); }
void orc_beads_move(void* h) {
  Oracle* o = static_cast<Oracle*>(h);
  o->ypglb_prev = o->ypglb;
  o->beads_move();
}
int orc_beads_redistribute(void* h) { return static_cast<Oracle*>(h)->beads_redistribute(); }
void orc_beads_links(void* h) { static_cast<Oracle*>(h)->beads_links(); }
void orc_beads_filling(void* h) { static_cast<Oracle*>(h)->beads_filling(); }
void orc_macrovar(void* h) { static_cast<Oracle*>(h)->macrovar(); }
void orc_rhoupdat(void* h) { static_cast<Oracle*>(h)->rhoupdat(); }
void orc_initpop(void* h) { static_cast<Oracle*>(h)->initpop(); }
int orc_initpartpos(void* h, int np) { return static_cast<Oracle*>(h)->initpartpos(np); }
int orc_initpartvel(void* h, int np) { return static_cast<Oracle*>(h)->initpartvel(np); }
// positions already in ypglb (set through orc_field), velocities in wp/omgp
void orc_release(void* h, int np) { static_cast<Oracle*>(h)->release(np); }
// host threads of the parallel loops (the CPU baseline's core count)
void orc_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
void orc_restore(void* h, int np) { static_cast<Oracle*>(h)->restore(np); }
int orc_step(void* h, int nsteps) {
  Oracle* o = static_cast<Oracle*>(h);
  for (int s = 0; s < nsteps; ++s) {
    int rc = o->step();
    if (rc) return rc;
  }
  return 0;
}
// n successive ran1 draws from a fresh state seeded with -seed (for tests)
void orc_ran1_sequence(int32_t seed, int n, double* out) {
  int32_t idum = -seed, iy = 0, iv[32];
  std::memset(iv, 0, sizeof(iv));
  for (int i = 0; i < n; ++i) out[i] = ran1(&idum, &iy, iv);
}
// The Park-Miller state idum after n ran1 draws from a fresh state seeded
// with -seed: the core sequence x_{k+1} = 16807 x_k mod (2^31 - 1) from
// x_0 = seed, advanced by NTAB + 8 = 40 steps at the first draw (the shuffle
// table's warm-up) and one step per draw (for the known-answer tests).
int32_t orc_ran1_state(int32_t seed, int n) {
  int32_t idum = -seed, iy = 0, iv[32];
  std::memset(iv, 0, sizeof(iv));
  for (int i = 0; i < n; ++i) ran1(&idum, &iy, iv);
  return idum;
}
}
