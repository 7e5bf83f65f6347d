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

}  // namespace

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
  double* terms = nullptr;    // 3 N scratch (shell terms, moment terms)
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
      !al((void**)&w->terms, 3 * N * sizeof(double)) ||
      !al((void**)&w->sums, (2 * (size_t)w->nek + 8) * sizeof(double)))
    return LBM_ERR_NOMEM;
  cudaMemcpy(w->perm, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(w->offsets, off.data(), off.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  size_t b1 = 0, b2 = 0;
  cub::DeviceSegmentedReduce::Sum(nullptr, b1, w->terms, w->sums, w->nek, w->offsets,
                                  w->offsets + 1);
  cub::DeviceReduce::Sum(nullptr, b2, w->terms, w->sums, N);
  w->cub_bytes = b1 > b2 ? b1 : b2;
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
  template void launch_slip<T>(const Geometry&, const ParticleView&, const T*, const T*,      \
                               const T*, const int32_t*, double, double, double*, cudaStream_t);
LBM_STATS_INSTANTIATE(float)
LBM_STATS_INSTANTIATE(double)

}  // namespace lbm
