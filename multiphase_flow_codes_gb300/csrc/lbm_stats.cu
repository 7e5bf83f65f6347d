// lbm_stats.cu - flow statistics on the device: the energy spectrum,
// dissipation rate and velocity-derivative moments of statistc
// (B/saveload.f90:1111-1338), and the slip velocity of each particle.
//
// statistc transforms the velocity with a forward FFT normalised by 1/N per
// axis (B/mpifft.f90:52-108), sums |u^(k)|^2 over the half spectrum kx >= 0
// with the kx = 0 plane weighted 1/2 into shells ik = int(|k| + 1/2),
// ik = 1 .. nek, nek = int(nx/2 - 1.5) (B/para.f90:83, gaussian.f90:73), and
// the dissipation 2 nu k^2 E in the same shells.  Here the FFTs are cuFFT
// double-precision transforms (the library's, not a hand-written one: the
// statistics are off the time step's hot path), the shell sums are
// deterministic segmented reductions over a mode permutation sorted by
// shell, and the dissipation includes (2 pi / n)^2 per axis so that it is in
// lattice units (the reference folds that factor into dscale,
// B/para.f90:47-59).
//
// The skewness and flatness follow statistc's own formula, including its
// use of wx where wz would be expected (B/saveload.f90:1181-1193):
//   S = <(wx^3 + wy^3 + wx^3) / 3> / <(wx^2 + wy^2 + wx^2) / 3>^1.5,
// with w_a = d u_a / d x_a from the spectral derivative.
#include <cub/cub.cuh>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "lbm_internal.cuh"

namespace lbm {

namespace {

__device__ __forceinline__ int signed_k(int i, int n) { return i <= n / 2 ? i : i - n; }

// |u^|^2 contributions of each mode, gathered in shell order
__global__ void k_shell_terms(int nx, int ny, int nz, const double2* __restrict__ vx,
                              const double2* __restrict__ vy, const double2* __restrict__ vz,
                              const int32_t* __restrict__ perm, long long nperm, double inv_n2,
                              double two_nu, double* __restrict__ e, double* __restrict__ d) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nperm) return;
  const int m = perm[t];
  const int nxc = nx / 2 + 1;
  const int kx = m % nxc;
  const int r = m / nxc;
  const int ky = signed_k(r % ny, ny), kz = signed_k(r / ny, nz);
  const double2 a = vx[m], b = vy[m], c = vz[m];
  double s = (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y) * inv_n2;
  if (kx == 0) s *= 0.5;
  const double pi2 = 6.283185307179586;
  const double qx = pi2 * kx / nx, qy = pi2 * ky / ny, qz = pi2 * kz / nz;
  e[t] = s;
  d[t] = two_nu * (qx * qx + qy * qy + qz * qz) * s;
}

// spectral derivative w_a = d u_a / d x_a: multiply by i k_a (integer k, as
// statistc does; the moments are ratios, so the 2 pi / n factor cancels).
// The Nyquist wavenumber of each axis is dropped so that w_a is a real
// field whatever the inverse transform does with non-Hermitian input.
__global__ void k_derivative(int nx, int ny, int nz, double2* vx, double2* vy, double2* vz,
                             double inv_n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nxc = nx / 2 + 1;
  const long long total = (long long)nxc * ny * nz;
  if (t >= total) return;
  const int kx = (int)(t % nxc);
  const long long r = t / nxc;
  const int ky = signed_k((int)(r % ny), ny), kz = signed_k((int)(r / ny), nz);
  double2* v[3] = {vx, vy, vz};
  const int k[3] = {2 * kx == nx ? 0 : kx, 2 * ky == ny ? 0 : ky, 2 * kz == nz ? 0 : kz};
  for (int a = 0; a < 3; ++a) {
    const double2 u = v[a][t];
    v[a][t] = make_double2(-k[a] * u.y * inv_n, k[a] * u.x * inv_n);
  }
}

// per node the statistc moments p = 2, 3, 4 of (wx, wy, wx)
__global__ void k_moment_terms(long long n, const double* __restrict__ wx,
                               const double* __restrict__ wy, double* __restrict__ m2,
                               double* __restrict__ m3, double* __restrict__ m4) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double a = wx[t], b = wy[t];
  const double a2 = a * a, b2 = b * b;
  m2[t] = (a2 + b2 + a2) / 3.0;
  m3[t] = (a2 * a + b2 * b + a2 * a) / 3.0;
  m4[t] = (a2 * a2 + b2 * b2 + a2 * a2) / 3.0;
}

template <typename T>
__global__ void k_to_double(const T* __restrict__ in, double* __restrict__ out, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = (double)in[t];
}

__device__ __forceinline__ double nearest(double d, int n) {
  if (d > 0.5 * n) return d - n;
  if (d < -0.5 * n) return d + n;
  return d;
}

// Slip of particle p: w_p minus the mean fluid velocity over the fluid nodes
// at distance r_in <= r <= r_out from the centre (nearest periodic image).
// One block per particle, fixed-order reduction.  Each axis walks the window
// of 2 h + 1 nodes around the centre, or the whole axis when that is
// shorter, so every node is visited once.
template <typename T>
__global__ void __launch_bounds__(256) k_slip(Geometry g, ParticleView pv, const T* __restrict__ ux,
                                              const T* __restrict__ uy, const T* __restrict__ uz,
                                              const int32_t* __restrict__ isnodes, double r_in,
                                              double r_out, double* __restrict__ slip) {
  using Red = cub::BlockReduce<double, 256>;
  __shared__ typename Red::TempStorage tmp;
  const int p = blockIdx.x;
  if (p >= pv.npart) return;
  const double xc = pv.ypglb[3 * p], yc = pv.ypglb[3 * p + 1], zc = pv.ypglb[3 * p + 2];
  const int h = (int)ceil(r_out) + 1;
  // node (i, j, k) (0-based) sits at (i + 1/2, j + 1/2, k + 1/2)
  const int wx = min(2 * h + 1, g.nx), wy = min(2 * h + 1, g.ny), wz = min(2 * h + 1, g.nz);
  const int i0 = wx < g.nx ? (int)floor(xc - 0.5) - h : 0;
  const int j0 = wy < g.ny ? (int)floor(yc - 0.5) - h : 0;
  const int k0 = wz < g.nz ? (int)floor(zc - 0.5) - h : 0;
  const long long box = (long long)wx * wy * wz;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long t = threadIdx.x; t < box; t += blockDim.x) {
    const int di = (int)(t % wx), dj = (int)((t / wx) % wy), dk = (int)(t / ((long long)wx * wy));
    int i = i0 + di;
    if (g.channel && (i < 0 || i >= g.nx)) continue;
    i = ((i % g.nx) + g.nx) % g.nx;
    const int j = (((j0 + dj) % g.ny) + g.ny) % g.ny;
    const int k = (((k0 + dk) % g.nz) + g.nz) % g.nz;
    const double dx = g.channel ? (i + 0.5 - xc) : nearest(i + 0.5 - xc, g.nx);
    const double dy = nearest(j + 0.5 - yc, g.ny), dz = nearest(k + 0.5 - zc, g.nz);
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < r_in * r_in || r2 > r_out * r_out) continue;
    const long long n = (long long)i + (long long)g.nx * (j + (long long)g.ny * k);
    if (isnodes[n] >= 0) continue;  // solid
    s[0] += (double)ux[n];
    s[1] += (double)uy[n];
    s[2] += (double)uz[n];
    s[3] += 1.0;
  }
  double tot[4];
  for (int c = 0; c < 4; ++c) {
    tot[c] = Red(tmp).Sum(s[c]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double cnt = tot[3] > 0.0 ? tot[3] : 1.0;
    for (int c = 0; c < 3; ++c) slip[3 * p + c] = pv.wp[3 * p + c] - tot[c] / cnt;
  }
}

inline unsigned blocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// ---- seeded solenoidal initial velocity --------------------------------
// counter-based generator: a splitmix64 hash of (seed, counter)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double unit_open(uint64_t h) {  // (0, 1]
  return ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}
// standard complex Gaussian of (seed, mode, component) by Box-Muller
__device__ __forceinline__ double2 gauss2(uint64_t seed, long long mode, int comp) {
  const uint64_t h1 = mix64(seed ^ mix64((uint64_t)mode * 8 + 2 * comp));
  const uint64_t h2 = mix64(seed ^ mix64((uint64_t)mode * 8 + 2 * comp + 1));
  const double r = sqrt(-2.0 * log(unit_open(h1)));
  const double t = 6.283185307179586 * unit_open(h2);
  return make_double2(r * cos(t), r * sin(t));
}

// Half-spectrum coefficients (kx >= 0) of a divergence-free Gaussian field,
// in the steps of the reference's initvel (3DBox.../initial.f90:55-116):
// per mode a complex Gaussian vector projected off k (tmp = k.v / k^2,
// v = v - k tmp), the kx = 0 plane made Hermitian (a mode and its mirror -k
// share one draw, conjugated; symmetrize, gaussian.f90:80-), the mean and
// the Nyquist wavenumbers of each axis set to zero (symmetrize), and the
// modes of shells beyond nek = int(nx/2 - 1.5) set to zero (initial.f90:77-81).
// The amplitude sqrt(E(k) / (4 pi k^2)) only pre-shapes the draw: the shell
// energies are set exactly afterwards (k_shell_energy, k_shell_scale).
__global__ void k_spectral_modes(int nx, int ny, int nz, double k0, uint64_t seed,
                                 double2* __restrict__ vx, double2* __restrict__ vy,
                                 double2* __restrict__ vz) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nxc = nx / 2 + 1;
  const long long total = (long long)nxc * ny * nz;
  if (t >= total) return;
  const int kx = (int)(t % nxc);
  const long long r = t / nxc;
  int jy = (int)(r % ny), jz = (int)(r / ny);
  int ky = signed_k(jy, ny), kz = signed_k(jz, nz);
  const double k2 = (double)kx * kx + (double)ky * ky + (double)kz * kz;
  const int nek = (int)(nx / 2 - 1.5);
  if (k2 == 0.0 || 2 * kx == nx || 2 * jy == ny || 2 * jz == nz ||
      (int)(sqrt(k2) + 0.5) > nek) {
    vx[t] = vy[t] = vz[t] = make_double2(0.0, 0.0);
    return;
  }
  // Hermitian planes: draw from the canonical member of the pair (k, -k)
  bool conj = false;
  if (kx == 0 || 2 * kx == nx) {
    const int my = (ny - jy) % ny, mz = (nz - jz) % nz;  // index of -k
    if (my > jy || (my == jy && mz > jz)) {
      conj = true;
      jy = my;
      jz = mz;
      ky = signed_k(jy, ny);
      kz = signed_k(jz, nz);
    }
  }
  const long long canon = ((long long)jz * ny + jy) * nxc + kx;
  double2 a[3] = {gauss2(seed, canon, 0), gauss2(seed, canon, 1), gauss2(seed, canon, 2)};
  const double kv[3] = {(double)kx, (double)ky, (double)kz};
  // solenoidal projection a - k (k.a) / k^2, real and imaginary parts
  const double kr = (kv[0] * a[0].x + kv[1] * a[1].x + kv[2] * a[2].x) / k2;
  const double ki = (kv[0] * a[0].y + kv[1] * a[1].y + kv[2] * a[2].y) / k2;
  const double k = sqrt(k2), q = k / k0;
  const double amp = sqrt(k2 * k2 * exp(-2.0 * q * q) / (4.0 * 3.141592653589793 * k2));
  double2 out[3];
  for (int c = 0; c < 3; ++c) {
    out[c] = make_double2(amp * (a[c].x - kv[c] * kr), amp * (a[c].y - kv[c] * ki));
    if (conj) out[c].y = -out[c].y;
  }
  // self-mirror modes (k = -k on the grid) must be real
  if ((kx == 0 || 2 * kx == nx) && ((ny - jy) % ny) == jy && ((nz - jz) % nz) == jz)
    for (int c = 0; c < 3; ++c) out[c].y = 0.0;
  vx[t] = out[0];
  vy[t] = out[1];
  vz[t] = out[2];
}

// Target energy of shell ik: the workload's spectrum ik^4 exp(-2 (ik/k0)^2)
__device__ __forceinline__ double shell_target(int ik, double k0) {
  const double q = (double)ik / k0;
  return (double)ik * ik * ik * ik * exp(-2.0 * q * q);
}

// Energy of every shell int(|k| + 1/2) = 1..nek over the half spectrum, the
// kx = 0 plane weighted 1/2 as initvel and statistc count it, relative to the
// shell's target energy.  Each mode's share is converted to 64-bit fixed
// point at 2^-kShellFx and added with integer atomics, per block in shared
// memory and then per shell in global memory: integer addition does not
// depend on the order, so the sums are the same bits on every run.  (The
// modes are pre-shaped to the target spectrum, so a shell sums to a few
// units whatever its energy.)
constexpr int kShellFx = 50;
__global__ void __launch_bounds__(256) k_shell_energy(int nx, int ny, int nz, double k0,
                                                      const double2* __restrict__ vx,
                                                      const double2* __restrict__ vy,
                                                      const double2* __restrict__ vz,
                                                      unsigned long long* __restrict__ acc) {
  extern __shared__ unsigned long long sacc[];
  const int nek = (int)(nx / 2 - 1.5);
  for (int i = threadIdx.x; i <= nek; i += blockDim.x) sacc[i] = 0ull;
  __syncthreads();
  const int nxc = nx / 2 + 1;
  const long long total = (long long)nxc * ny * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(t % nxc);
    const long long r = t / nxc;
    const int ky = signed_k((int)(r % ny), ny), kz = signed_k((int)(r / ny), nz);
    const double k2 = (double)kx * kx + (double)ky * ky + (double)kz * kz;
    const int ik = (int)(sqrt(k2) + 0.5);
    if (ik < 1 || ik > nek) continue;
    const double target = shell_target(ik, k0);
    if (!(target > 0.0)) continue;
    const double2 a = vx[t], b = vy[t], c = vz[t];
    double e = a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y;
    if (kx == 0) e *= 0.5;
    const double q = ldexp(e / target, kShellFx);
    atomicAdd(&sacc[ik], (unsigned long long)llrint(fmin(q, 9.0e18)));
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= nek; i += blockDim.x)
    if (sacc[i]) atomicAdd(&acc[i], sacc[i]);
}

// Scale every mode of shell ik so that the shell holds its target energy
// (initvel's per-shell rescaling with the workload's spectrum).
__global__ void k_shell_scale(int nx, int ny, int nz,
                              const unsigned long long* __restrict__ acc,
                              double2* __restrict__ vx, double2* __restrict__ vy,
                              double2* __restrict__ vz) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nxc = nx / 2 + 1;
  const long long total = (long long)nxc * ny * nz;
  if (t >= total) return;
  const int kx = (int)(t % nxc);
  const long long r = t / nxc;
  const int ky = signed_k((int)(r % ny), ny), kz = signed_k((int)(r / ny), nz);
  const double k2 = (double)kx * kx + (double)ky * ky + (double)kz * kz;
  const int ik = (int)(sqrt(k2) + 0.5);
  const int nek = (int)(nx / 2 - 1.5);
  double f = 0.0;
  if (ik >= 1 && ik <= nek && acc[ik] > 0ull)
    f = sqrt(1.0 / ldexp((double)acc[ik], -kShellFx));  // sqrt(target / shell energy)
  vx[t] = make_double2(vx[t].x * f, vx[t].y * f);
  vy[t] = make_double2(vy[t].x * f, vy[t].y * f);
  vz[t] = make_double2(vz[t].x * f, vz[t].y * f);
}

__global__ void k_square(const double* __restrict__ a, double* __restrict__ b, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) b[t] = a[t] * a[t];
}
// The channel's initial velocity, initvel of 3DChannel.../initial.f90:57-126:
// walls normal to x at x = 0 and x = nx, u = w = 0, and the mean profile
// v(x) = y+ ustar in the viscous sublayer (y+ < 10.8) and (ln(y+)/0.41 + 5)
// ustar beyond it, y+ = (i - 1/2) / ystar for the nx/2 nodes nearest each
// wall (a middle node of an odd nx keeps 0).  The reference's perturbation
// terms carry the amplitude A9 = 0 and vanish.
__global__ void k_channel_loglaw(int nx, long long N, double ustar, double ystar,
                                 double* __restrict__ u) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int i = (int)(t % nx) + 1;  // 1-based wall-normal index
  const int nxh = nx / 2;
  const int ii = i <= nxh ? i : nx + 1 - i;
  double v = 0.0;
  if (ii <= nxh) {
    const double yplus = ((double)ii - 0.5) / ystar;
    if (yplus < 10.8) {
      v = yplus * ustar;
    } else {
      double u9 = log(yplus) / 0.41 + 5.0;
      v = u9 * ustar;
    }
  }
  u[t] = 0.0;
  u[N + t] = v;
  u[2 * N + t] = 0.0;
}

// u *= urms / sqrt(sum of squares / count): one factor for all components
__global__ void k_scale(double* __restrict__ a, long long n, const double* __restrict__ sumsq,
                        double count, double urms) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) {
    const double ms = *sumsq / count;
    a[t] = ms > 0.0 ? a[t] * (urms / sqrt(ms)) : 0.0;
  }
}

// Deterministic summary of a state: per block partial sums of mass, x/y/z
// momentum, a position-weighted population checksum, and (from the macro
// arrays) the kinetic energy.
template <typename T>
__global__ void __launch_bounds__(256) k_summary(const T* __restrict__ f, long long N,
                                                 const T* __restrict__ ux, const T* __restrict__ uy,
                                                 const T* __restrict__ uz,
                                                 double* __restrict__ partial) {
  using Red = cub::BlockReduce<double, 256>;
  __shared__ typename Red::TempStorage tmp;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N;
       n += (long long)gridDim.x * blockDim.x) {
    double rho = 0.0, jx = 0.0, jy = 0.0, jz = 0.0, ck = 0.0;
#pragma unroll
    for (int q = 0; q < NPOP; ++q) {
      const double v = (double)f[(long long)q * N + n];
      rho += v;
      jx += cix(q) * v;
      jy += ciy(q) * v;
      jz += ciz(q) * v;
      ck += (1.0 + q / 19.0 + (double)(n % 97) / 97.0) * v;
    }
    s[0] += rho; s[1] += jx; s[2] += jy; s[3] += jz; s[4] += ck;
    const double a = (double)ux[n], b = (double)uy[n], c = (double)uz[n];
    s[5] += 0.5 * (a * a + b * b + c * c);
  }
  for (int c = 0; c < 6; ++c) {
    const double t = Red(tmp).Sum(s[c]);
    __syncthreads();
    if (threadIdx.x == 0) partial[6 * blockIdx.x + c] = t;
  }
}

}  // namespace

int spectral_field(const Geometry& g, double k0, double urms, uint64_t seed, double* u,
                   cudaStream_t s) {
  const long long N = g.N;
  const long long nc = (long long)(g.nx / 2 + 1) * g.ny * g.nz;
  const int nek = (int)(g.nx / 2 - 1.5);
  double2* spec = nullptr;
  double* tmp = nullptr;
  unsigned long long* shell_acc = nullptr;
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
  cufftHandle plan = 0;
  int rc = LBM_OK;
  cub::DeviceReduce::Sum(nullptr, cub_bytes, tmp, tmp, 3 * N);
  if (cudaMalloc((void**)&spec, 3 * nc * sizeof(double2)) != cudaSuccess ||
      cudaMalloc((void**)&tmp, (3 * N + 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&shell_acc, (nek + 2) * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&cub_tmp, cub_bytes) != cudaSuccess) {
    rc = LBM_ERR_NOMEM;
  } else if (cufftPlan3d(&plan, g.nz, g.ny, g.nx, CUFFT_Z2D) != CUFFT_SUCCESS) {
    rc = LBM_ERR_CUDA;
    plan = 0;
  } else {
    cufftSetStream(plan, s);
    k_spectral_modes<<<blocks(nc, 256), 256, 0, s>>>(g.nx, g.ny, g.nz, k0, seed, spec,
                                                      spec + nc, spec + 2 * nc);
    count_launch();
    if (nek >= 1) {
      cudaMemsetAsync(shell_acc, 0, (nek + 2) * sizeof(unsigned long long), s);
      const unsigned grid = (unsigned)std::min<long long>(blocks(nc, 256), 8LL * sm_count());
      k_shell_energy<<<grid, 256, (nek + 1) * sizeof(unsigned long long), s>>>(
          g.nx, g.ny, g.nz, k0, spec, spec + nc, spec + 2 * nc, shell_acc);
      count_launch();
      k_shell_scale<<<blocks(nc, 256), 256, 0, s>>>(g.nx, g.ny, g.nz, shell_acc, spec, spec + nc,
                                                    spec + 2 * nc);
      count_launch();
    }
    for (int c = 0; c < 3 && !rc; ++c)
      if (cufftExecZ2D(plan, spec + c * nc, u + c * N) != CUFFT_SUCCESS) rc = LBM_ERR_CUDA;
    if (!rc) {
      // one factor for all three components, so the field stays solenoidal:
      // sqrt(mean |u|^2 / 3) -> urms
      k_square<<<blocks(3 * N, 256), 256, 0, s>>>(u, tmp, 3 * N);
      count_launch();
      size_t b = cub_bytes;
      cub::DeviceReduce::Sum(cub_tmp, b, tmp, tmp + 3 * N, 3 * N, s);
      k_scale<<<blocks(3 * N, 256), 256, 0, s>>>(u, 3 * N, tmp + 3 * N, (double)(3 * N), urms);
      count_launch();
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = LBM_ERR_CUDA;
  if (plan) cufftDestroy(plan);
  cudaFree(spec);
  cudaFree(tmp);
  cudaFree(shell_acc);
  cudaFree(cub_tmp);
  return rc;
}

int channel_loglaw_field(const Geometry& g, double visc, double* u, cudaStream_t s) {
  const double rstar = 180.0;                       // 3DChannel.../para.f90:14
  const double ustar = 2.0 * rstar * visc / (double)g.nx;
  const double ystar = visc / ustar;
  k_channel_loglaw<<<blocks(g.N, 256), 256, 0, s>>>(g.nx, g.N, ustar, ystar, u);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

template <typename T>
void launch_summary(const T* f, long long N, const T* ux, const T* uy, const T* uz,
                    double* partial, int nblocks, cudaStream_t s) {
  k_summary<T><<<nblocks, 256, 0, s>>>(f, N, ux, uy, uz, partial);
  count_launch();
}

// ---------------------------------------------------------------------------
struct SpectrumWork {
  int nx = 0, ny = 0, nz = 0, nek = 0;
  cufftHandle fwd = 0, inv = 0;
  bool plans = false;
  double* real = nullptr;     // 3 N doubles (input copies / derivative fields)
  double2* spec = nullptr;    // 3 (nx/2+1) ny nz
  int32_t* perm = nullptr;    // modes of shells 1..nek, sorted by shell
  long long nperm = 0;
  int32_t* offsets = nullptr; // nek + 1 segment offsets
  double* terms = nullptr;    // 4 N scratch (shell, moment and masked terms)
  double* sums = nullptr;     // results
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
};

void spectrum_free(SpectrumWork* w) {
  if (!w) return;
  if (w->plans) {
    cufftDestroy(w->fwd);
    cufftDestroy(w->inv);
  }
  cudaFree(w->real);
  cudaFree(w->spec);
  cudaFree(w->perm);
  cudaFree(w->offsets);
  cudaFree(w->terms);
  cudaFree(w->sums);
  cudaFree(w->cub_tmp);
  delete w;
}

static int spectrum_setup(const Geometry& g, SpectrumWork** pw) {
  if (*pw) return LBM_OK;
  SpectrumWork* w = new SpectrumWork();
  *pw = w;
  w->nx = g.nx; w->ny = g.ny; w->nz = g.nz;
  w->nek = (int)(g.nx / 2 - 1.5);
  const long long N = g.N;
  const long long nc = (long long)(g.nx / 2 + 1) * g.ny * g.nz;
  if (cufftPlan3d(&w->fwd, g.nz, g.ny, g.nx, CUFFT_D2Z) != CUFFT_SUCCESS) return LBM_ERR_CUDA;
  if (cufftPlan3d(&w->inv, g.nz, g.ny, g.nx, CUFFT_Z2D) != CUFFT_SUCCESS) {
    cufftDestroy(w->fwd);
    return LBM_ERR_CUDA;
  }
  w->plans = true;
  // mode permutation: stable counting sort of the half-spectrum modes by
  // shell int(|k| + 1/2), keeping shells 1 .. nek
  std::vector<int> count(w->nek + 2, 0);
  std::vector<int32_t> shell(nc);
  const int nxc = g.nx / 2 + 1;
  for (long long m = 0; m < nc; ++m) {
    const int kx = (int)(m % nxc);
    const long long r = m / nxc;
    int ky = (int)(r % g.ny), kz = (int)(r / g.ny);
    if (ky > g.ny / 2) ky -= g.ny;
    if (kz > g.nz / 2) kz -= g.nz;
    const int ik = (int)(std::sqrt((double)kx * kx + (double)ky * ky + (double)kz * kz) + 0.5);
    shell[m] = (ik >= 1 && ik <= w->nek) ? ik : 0;
    if (shell[m]) ++count[ik];
  }
  std::vector<int32_t> off(w->nek + 1, 0);
  for (int ik = 1; ik <= w->nek; ++ik) off[ik] = off[ik - 1] + count[ik];
  w->nperm = off[w->nek];
  std::vector<int32_t> perm(w->nperm > 0 ? w->nperm : 1);
  std::vector<int32_t> pos(off.begin(), off.end());
  for (long long m = 0; m < nc; ++m)
    if (shell[m]) perm[pos[shell[m] - 1]++] = (int32_t)m;
  auto al = [](void** p, size_t b) { return cudaMalloc(p, b) == cudaSuccess; };
  if (!al((void**)&w->real, 3 * N * sizeof(double)) ||
      !al((void**)&w->spec, 3 * nc * sizeof(double2)) ||
      !al((void**)&w->perm, perm.size() * sizeof(int32_t)) ||
      !al((void**)&w->offsets, off.size() * sizeof(int32_t)) ||
      !al((void**)&w->terms, 4 * N * sizeof(double)) ||
      !al((void**)&w->sums, (2 * (size_t)w->nek + 8) * sizeof(double)))
    return LBM_ERR_NOMEM;
  cudaMemcpy(w->perm, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(w->offsets, off.data(), off.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  size_t b1 = 0, b2 = 0;
  cub::DeviceSegmentedReduce::Sum(nullptr, b1, w->terms, w->sums, w->nek, w->offsets,
                                  w->offsets + 1);
  cub::DeviceReduce::Sum(nullptr, b2, w->terms, w->sums, N);
  size_t b3 = 0;
  cub::DeviceReduce::Max(nullptr, b3, w->terms, w->sums, N);
  w->cub_bytes = std::max(b1, std::max(b2, b3));
  if (!al(&w->cub_tmp, w->cub_bytes)) return LBM_ERR_NOMEM;
  return cudaGetLastError() == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

template <typename T>
int spectrum_stats(const Geometry& g, double visc, const T* ux, const T* uy, const T* uz,
                   SpectrumWork** pw, int nek_out, double* ek, double* dk, double* out,
                   cudaStream_t s) {
  if (int rc = spectrum_setup(g, pw)) return rc;
  SpectrumWork* w = *pw;
  const long long N = g.N;
  const long long nc = (long long)(g.nx / 2 + 1) * g.ny * g.nz;
  const T* u[3] = {ux, uy, uz};
  for (int a = 0; a < 3; ++a) {
    k_to_double<T><<<blocks(N, 256), 256, 0, s>>>(u[a], w->real + a * N, N);
    count_launch();
  }
  cufftSetStream(w->fwd, s);
  cufftSetStream(w->inv, s);
  for (int a = 0; a < 3; ++a)
    if (cufftExecD2Z(w->fwd, w->real + a * N, w->spec + a * nc) != CUFFT_SUCCESS) return LBM_ERR_CUDA;
  const double inv_n = 1.0 / (double)N;
  if (w->nperm > 0) {
    k_shell_terms<<<blocks(w->nperm, 256), 256, 0, s>>>(g.nx, g.ny, g.nz, w->spec, w->spec + nc,
                                                        w->spec + 2 * nc, w->perm, w->nperm,
                                                        inv_n * inv_n, 2.0 * visc, w->terms,
                                                        w->terms + w->nperm);
    count_launch();
    size_t b = w->cub_bytes;
    cub::DeviceSegmentedReduce::Sum(w->cub_tmp, b, w->terms, w->sums, w->nek, w->offsets,
                                    w->offsets + 1, s);
    b = w->cub_bytes;
    cub::DeviceSegmentedReduce::Sum(w->cub_tmp, b, w->terms + w->nperm, w->sums + w->nek, w->nek,
                                    w->offsets, w->offsets + 1, s);
  }
  // derivative moments
  k_derivative<<<blocks(nc, 256), 256, 0, s>>>(g.nx, g.ny, g.nz, w->spec, w->spec + nc,
                                               w->spec + 2 * nc, inv_n);
  count_launch();
  for (int a = 0; a < 2; ++a)  // statistc uses wx and wy only
    if (cufftExecZ2D(w->inv, w->spec + a * nc, w->real + a * N) != CUFFT_SUCCESS) return LBM_ERR_CUDA;
  k_moment_terms<<<blocks(N, 256), 256, 0, s>>>(N, w->real, w->real + N, w->terms,
                                                w->terms + N, w->terms + 2 * N);
  count_launch();
  for (int p = 0; p < 3; ++p) {
    size_t b = w->cub_bytes;
    cub::DeviceReduce::Sum(w->cub_tmp, b, w->terms + p * N, w->sums + 2 * w->nek + p, N, s);
  }
  std::vector<double> h(2 * (size_t)w->nek + 3);
  if (cudaMemcpyAsync(h.data(), w->sums, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LBM_ERR_CUDA;
  double qq = 0.0, dis = 0.0;
  for (int ik = 0; ik < w->nek; ++ik) {
    if (ik < nek_out) {
      if (ek) ek[ik] = h[ik];
      if (dk) dk[ik] = h[w->nek + ik];
    }
    qq += h[ik];
    dis += h[w->nek + ik];
  }
  const double cc2 = h[2 * w->nek] / N, cc3 = h[2 * w->nek + 1] / N, cc4 = h[2 * w->nek + 2] / N;
  out[0] = w->nek;
  out[1] = qq;
  out[2] = dis;
  out[3] = cc2 > 0 ? cc3 / pow(cc2, 1.5) : 0.0;
  out[4] = cc2 > 0 ? cc4 / (cc2 * cc2) : 0.0;
  out[5] = sqrt(2.0 * qq / 3.0);
  return LBM_OK;
}

// ---- rmsstat and diag (B/saveload.f90:1530-1730, 1342-1400) --------------

// fluid-masked terms of three fields: pass 0 the values (and a 1 per fluid
// node in t[3]), pass 1 the squared deviations from the means
__global__ void k_masked_terms(long long n, const int32_t* __restrict__ isnodes,
                               const double* __restrict__ a, const double* __restrict__ b,
                               const double* __restrict__ c, double ma, double mb, double mc,
                               int pass, double* __restrict__ t) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool fluid = isnodes[i] < 0;
  if (pass == 0) {
    t[i] = fluid ? a[i] : 0.0;
    t[n + i] = fluid ? b[i] : 0.0;
    t[2 * n + i] = fluid ? c[i] : 0.0;
    t[3 * n + i] = fluid ? 1.0 : 0.0;
  } else {
    const double da = a[i] - ma, db = b[i] - mb, dc = c[i] - mc;
    t[i] = fluid ? da * da : 0.0;
    t[n + i] = fluid ? db * db : 0.0;
    t[2 * n + i] = fluid ? dc * dc : 0.0;
  }
}

// vorticity o = curl u from the spectrum: i k x u^ (integer k as vortcalc
// uses, B/saveload.f90:3411-3450; Nyquist dropped as in k_derivative),
// normalised by 1/N for the unnormalised inverse
__global__ void k_curl(int nx, int ny, int nz, double2* vx, double2* vy, double2* vz,
                       double inv_n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nxc = nx / 2 + 1;
  const long long total = (long long)nxc * ny * nz;
  if (t >= total) return;
  const int kxi = (int)(t % nxc);
  const long long r = t / nxc;
  const int kyi = signed_k((int)(r % ny), ny), kzi = signed_k((int)(r / ny), nz);
  const double kx = 2 * kxi == nx ? 0 : kxi, ky = 2 * kyi == ny ? 0 : kyi,
               kz = 2 * kzi == nz ? 0 : kzi;
  const double2 a = vx[t], b = vy[t], c = vz[t];
  // w = k x u (complex), then times i: (re, im) -> (-im, re)
  const double2 wx = make_double2(ky * c.x - kz * b.x, ky * c.y - kz * b.y);
  const double2 wy = make_double2(kz * a.x - kx * c.x, kz * a.y - kx * c.y);
  const double2 wz = make_double2(kx * b.x - ky * a.x, kx * b.y - ky * a.y);
  vx[t] = make_double2(-wx.y * inv_n, wx.x * inv_n);
  vy[t] = make_double2(-wy.y * inv_n, wy.x * inv_n);
  vz[t] = make_double2(-wz.y * inv_n, wz.x * inv_n);
}

// |u| at fluid nodes, 0 at solid ones (diag's vel)
template <typename T>
__global__ void k_speed(long long n, const int32_t* __restrict__ isnodes, const T* __restrict__ ux,
                        const T* __restrict__ uy, const T* __restrict__ uz, double* __restrict__ v) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = ux[i], b = uy[i], c = uz[i];
  v[i] = isnodes[i] >= 0 ? 0.0 : sqrt(a * a + b * b + c * c);
}

// masked mean and rms of three double fields into m[3], rms[3]; nf counted
static int masked_mean_rms(SpectrumWork* w, long long N, const int32_t* isnodes, const double* a,
                           const double* b, const double* c, double* m, double* rms, long long* nf,
                           cudaStream_t s) {
  double h[4];
  k_masked_terms<<<blocks(N, 256), 256, 0, s>>>(N, isnodes, a, b, c, 0, 0, 0, 0, w->terms);
  count_launch();
  for (int k = 0; k < 4; ++k) {
    size_t bb = w->cub_bytes;
    cub::DeviceReduce::Sum(w->cub_tmp, bb, w->terms + k * N, w->sums + k, N, s);
  }
  if (cudaMemcpyAsync(h, w->sums, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LBM_ERR_CUDA;
  const long long n = (long long)h[3];
  *nf = n;
  for (int k = 0; k < 3; ++k) m[k] = n > 0 ? h[k] / (double)n : 0.0;
  k_masked_terms<<<blocks(N, 256), 256, 0, s>>>(N, isnodes, a, b, c, m[0], m[1], m[2], 1, w->terms);
  count_launch();
  for (int k = 0; k < 3; ++k) {
    size_t bb = w->cub_bytes;
    cub::DeviceReduce::Sum(w->cub_tmp, bb, w->terms + k * N, w->sums + k, N, s);
  }
  if (cudaMemcpyAsync(h, w->sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LBM_ERR_CUDA;
  for (int k = 0; k < 3; ++k) rms[k] = n > 0 ? sqrt(h[k] / (double)n) : 0.0;
  return LBM_OK;
}

template <typename T>
int fluid_rms_stats(const Geometry& g, const int32_t* isnodes, const T* ux, const T* uy,
                    const T* uz, SpectrumWork** pw, double* out, cudaStream_t s) {
  if (int rc = spectrum_setup(g, pw)) return rc;
  SpectrumWork* w = *pw;
  const long long N = g.N;
  const long long nc = (long long)(g.nx / 2 + 1) * g.ny * g.nz;
  const T* u[3] = {ux, uy, uz};
  for (int a = 0; a < 3; ++a) {
    k_to_double<T><<<blocks(N, 256), 256, 0, s>>>(u[a], w->real + a * N, N);
    count_launch();
  }
  long long nf = 0;
  double um[3], ur[3], om[3], orr[3];
  if (int rc = masked_mean_rms(w, N, isnodes, w->real, w->real + N, w->real + 2 * N, um, ur, &nf, s))
    return rc;
  // vortcalc: the whole velocity field, solid nodes included
  cufftSetStream(w->fwd, s);
  cufftSetStream(w->inv, s);
  for (int a = 0; a < 3; ++a)
    if (cufftExecD2Z(w->fwd, w->real + a * N, w->spec + a * nc) != CUFFT_SUCCESS) return LBM_ERR_CUDA;
  k_curl<<<blocks(nc, 256), 256, 0, s>>>(g.nx, g.ny, g.nz, w->spec, w->spec + nc, w->spec + 2 * nc,
                                         1.0 / (double)N);
  count_launch();
  for (int a = 0; a < 3; ++a)
    if (cufftExecZ2D(w->inv, w->spec + a * nc, w->real + a * N) != CUFFT_SUCCESS) return LBM_ERR_CUDA;
  long long nf2 = 0;
  if (int rc = masked_mean_rms(w, N, isnodes, w->real, w->real + N, w->real + 2 * N, om, orr, &nf2, s))
    return rc;
  out[0] = (double)nf;
  for (int k = 0; k < 3; ++k) {
    out[1 + k] = um[k];
    out[4 + k] = ur[k];
    out[7 + k] = om[k];
    out[10 + k] = orr[k];
  }
  return LBM_OK;
}

template <typename T>
int fluid_vmax(const Geometry& g, const int32_t* isnodes, const T* ux, const T* uy, const T* uz,
               SpectrumWork** pw, double* vmax, cudaStream_t s) {
  if (int rc = spectrum_setup(g, pw)) return rc;
  SpectrumWork* w = *pw;
  const long long N = g.N;
  k_speed<T><<<blocks(N, 256), 256, 0, s>>>(N, isnodes, ux, uy, uz, w->terms);
  count_launch();
  size_t bb = w->cub_bytes;
  cub::DeviceReduce::Max(w->cub_tmp, bb, w->terms, w->sums, N, s);
  if (cudaMemcpyAsync(vmax, w->sums, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LBM_ERR_CUDA;
  return LBM_OK;
}

// ---- wall-normal profiles of the channel's statistc / statistc2
// (C/saveload.f90:1136-1428): per x-plane sums over (y, z) of u, u_a u_b,
// rho, rho^2 and the fluid count.  Threads run along x (coalesced), blocks
// over chunks of kProfRows (y, z) rows; a second kernel adds the chunks in
// chunk order (deterministic).
constexpr int kProfRows = 64;
constexpr int kProfQ = 12;  // ux uy uz uxuz uxuy uyuz ux2 uy2 uz2 rho rho2 count

template <typename T>
__global__ void k_profile_partial(Geometry g, const int32_t* __restrict__ isnodes, int fluid_only,
                                  const T* __restrict__ rho, const T* __restrict__ ux,
                                  const T* __restrict__ uy, const T* __restrict__ uz,
                                  double* __restrict__ part) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= g.nx) return;
  const int nrows = g.ny * g.nz;
  const int r0 = blockIdx.y * kProfRows, r1 = min(nrows, r0 + kProfRows);
  double a[kProfQ];
#pragma unroll
  for (int q = 0; q < kProfQ; ++q) a[q] = 0.0;
  for (int r = r0; r < r1; ++r) {
    const long long n = (long long)r * g.nx + x;
    if (fluid_only && isnodes[n] >= 0) continue;
    const double u = ux[n], v = uy[n], w = uz[n], p = rho[n];
    a[0] += u; a[1] += v; a[2] += w;
    a[3] += u * w; a[4] += u * v; a[5] += v * w;
    a[6] += u * u; a[7] += v * v; a[8] += w * w;
    a[9] += p; a[10] += p * p; a[11] += 1.0;
  }
  double* o = part + ((long long)blockIdx.y * g.nx + x) * kProfQ;
#pragma unroll
  for (int q = 0; q < kProfQ; ++q) o[q] = a[q];
}

__global__ void k_profile_sum(int nx, int nchunks, const double* __restrict__ part,
                              double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // (x, q)
  if (t >= nx * kProfQ) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += part[(long long)c * nx * kProfQ + t];
  out[t] = s;
}

template <typename T>
int plane_sums(const Geometry& g, const int32_t* isnodes, int fluid_only, const T* rho,
               const T* ux, const T* uy, const T* uz, double* sums, cudaStream_t s) {
  const int nrows = g.ny * g.nz;
  const int nchunks = (nrows + kProfRows - 1) / kProfRows;
  double* d = nullptr;
  const size_t np = (size_t)nchunks * g.nx * kProfQ;
  if (cudaMalloc((void**)&d, (np + (size_t)g.nx * kProfQ) * sizeof(double)) != cudaSuccess)
    return LBM_ERR_NOMEM;
  k_profile_partial<T><<<dim3((g.nx + 127) / 128, nchunks), 128, 0, s>>>(g, isnodes, fluid_only, rho,
                                                                          ux, uy, uz, d);
  count_launch();
  k_profile_sum<<<blocks((long long)g.nx * kProfQ, 256), 256, 0, s>>>(g.nx, nchunks, d, d + np);
  count_launch();
  cudaError_t e = cudaMemcpyAsync(sums, d + np, (size_t)g.nx * kProfQ * sizeof(double),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  return e == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

template <typename T>
void launch_slip(const Geometry& g, const ParticleView& pv, const T* ux, const T* uy, const T* uz,
                 const int32_t* isnodes, double r_in, double r_out, double* slip, cudaStream_t s) {
  if (pv.npart <= 0) return;
  k_slip<T><<<pv.npart, 256, 0, s>>>(g, pv, ux, uy, uz, isnodes, r_in, r_out, slip);
  count_launch();
}

#define LBM_STATS_INSTANTIATE(T)                                                              \
  template int spectrum_stats<T>(const Geometry&, double, const T*, const T*, const T*,       \
                                 SpectrumWork**, int, double*, double*, double*, cudaStream_t); \
  template int fluid_rms_stats<T>(const Geometry&, const int32_t*, const T*, const T*,        \
                                  const T*, SpectrumWork**, double*, cudaStream_t);           \
  template int fluid_vmax<T>(const Geometry&, const int32_t*, const T*, const T*, const T*,    \
                             SpectrumWork**, double*, cudaStream_t);                          \
  template int plane_sums<T>(const Geometry&, const int32_t*, int, const T*, const T*,        \
                             const T*, const T*, double*, cudaStream_t);                      \
  template void launch_slip<T>(const Geometry&, const ParticleView&, const T*, const T*,      \
                               const T*, const int32_t*, double, double, double*, cudaStream_t); \
  template void launch_summary<T>(const T*, long long, const T*, const T*, const T*, double*,  \
                                  int, cudaStream_t);
LBM_STATS_INSTANTIATE(float)
LBM_STATS_INSTANTIATE(double)

}  // namespace lbm
