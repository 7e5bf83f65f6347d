// lbm_forcing.cu - device-side FORCING state update (B/gaussian.f90:182-307).
//
// The stochastic forcing draws 450 uniform numbers per call from a
// Park-Miller / Bays-Durham generator (ranff, B/gaussian.f90:374-404), turns
// them into complex white noise on the 6x5x5 low-mode block, advances the
// Ornstein-Uhlenbeck coefficients b1r..b3r and projects them onto
// divergence-free modes a1r..a3r.  Only the integer generator is sequential;
// one block runs the whole update on the device, so time steps need no host
// round trip (and can run inside CUDA graphs).  The generator is exact;
// compiled with -fmad=false, the floating-point updates round like the CPU
// restatement except where the device log/cos/sin differ from the host's by
// an ulp.
#include "lbm_internal.cuh"

namespace lbm {

namespace {

__device__ double ran1_dev(int32_t* idum, int32_t* iy, int32_t* iv) {
  const int32_t IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, NTAB = 32;
  const int32_t NDIV = 1 + (IM - 1) / NTAB;
  const double AM = 1.0 / IM, EPS = 1.2e-7, RNMX = 1.0 - EPS;
  int32_t k;
  if (*idum <= 0 || *iy == 0) {
    *idum = max(-*idum, 1);
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
  int32_t j = *iy / NDIV;
  *iy = iv[j];
  iv[j] = *idum;
  return fmin(AM * (double)(*iy), RNMX);
}

__device__ __forceinline__ int m655(int i, int j, int k) { return (i - 1) + 6 * (j - 1) + 30 * (k - 1); }

// a * b mod (2^31 - 1) for a, b in [1, 2^31 - 2], exact (2^31 = 1 mod m)
__device__ __forceinline__ int32_t mulmod_m31(int32_t a, int32_t b) {
  const unsigned long long p = (unsigned long long)(uint32_t)a * (uint32_t)b;
  unsigned long long r = (p & 0x7fffffffULL) + (p >> 31);
  r = (r & 0x7fffffffULL) + (r >> 31);
  if (r >= 0x7fffffffULL) r -= 0x7fffffffULL;
  return (int32_t)r;
}

// 16807^n mod (2^31 - 1): n steps of the generator's multiplier at once
__device__ __forceinline__ int32_t lcg_jump(int n) {
  int32_t r = 1, b = 16807;
  while (n) {
    if (n & 1) r = mulmod_m31(r, b);
    b = mulmod_m31(b, b);
    n >>= 1;
  }
  return r;
}

// One block.  The 450 uniform numbers come in the reference's order (mc, k,
// j, i = 1,3,5; cont1 then rph).  Their multiplicative congruential part is
// computed for all draws at once by jumping ahead (Schrage's form in ran1 is
// the exact product 16807 idum mod 2^31-1, so the jump gives the same
// integers); only the shuffle table's chain (iy selects the slot that the
// next idum replaces) runs in one thread, on shared memory.  The first call
// of a generator (idum <= 0: table initialisation) runs ran1 itself.  Then
// the magnitudes, phases, Ornstein-Uhlenbeck update and projection run one
// mode per thread on shared copies of the state.
__device__ __forceinline__ void k_forcing_update_body(int bx, int gx, ForcingDev* st, double var, double tf,
                                                        double pi2, const double* kxr6,
                                                        const double* kyr5, const double* kzr5) {
  __shared__ double u[450];
  __shared__ double fr[450];
  __shared__ double sb[450];
  __shared__ double sa[450];
  __shared__ int32_t lcg[450];
  __shared__ int32_t iys[450];
  __shared__ int32_t siv[32];
  __shared__ int32_t sstate[2];
  const int tid = threadIdx.x;
  const double smallx = 1.0e-18;
  const double xkf = sqrt(8.0);
  const double dt = 1.0;
  const double AM = 1.0 / 2147483647.0, RNMX = 1.0 - 1.2e-7;
  const int32_t idum0 = st->iseedf, iy0 = st->iyf;
  const bool init = idum0 <= 0 || iy0 == 0;  // the same in every thread
  if (tid < 32) siv[tid] = st->ivf[tid];
  for (int m = tid; m < 450; m += blockDim.x) sb[m] = st->b[m];
  if (!init)
    for (int n = tid; n < 450; n += blockDim.x) lcg[n] = mulmod_m31(idum0, lcg_jump(n + 1));
  __syncthreads();
  if (tid == 0) {
    if (init) {
      int32_t idum = idum0, iy = iy0;
      int32_t iv[32];
      for (int i = 0; i < 32; ++i) iv[i] = siv[i];
      for (int d = 0; d < 450; ++d) u[d] = ran1_dev(&idum, &iy, iv);
      for (int i = 0; i < 32; ++i) siv[i] = iv[i];
      sstate[0] = idum;
      sstate[1] = iy;
    } else {
      // ran1's shuffle: j = iy / NDIV with NDIV = 2^26 and iy >= 1
      int32_t iy = iy0;
      for (int d = 0; d < 450; ++d) {
        const int jj = iy >> 26;
        iy = siv[jj];
        siv[jj] = lcg[d];
        iys[d] = iy;
      }
      sstate[0] = lcg[449];
      sstate[1] = iy;
    }
  }
  __syncthreads();
  if (!init)
    for (int d = tid; d < 450; d += blockDim.x) u[d] = fmin(AM * (double)iys[d], RNMX);
  __syncthreads();
  // white noise, gaussian.f90:201-215; draw pair d <-> (mc, k, j, i)
  for (int d = tid; d < 225; d += blockDim.x) {
    int i = 1 + 2 * (d % 3);
    int r = d / 3;
    int j = 1 + r % 5; r /= 5;
    int k = 1 + r % 5;
    int mc = 1 + r / 5;
    double cont1 = u[2 * d];
    if (cont1 < 1.e-6) cont1 = 1.e-6;
    double rmag = sqrt(-4.0 * var * dt * log(cont1) / tf);
    double rph = u[2 * d + 1];
    fr[m655(i, j, k) + 150 * (mc - 1)] = rmag * cos(pi2 * rph);
    fr[m655(i + 1, j, k) + 150 * (mc - 1)] = rmag * sin(pi2 * rph);
  }
  __syncthreads();
  // real-valued forcing in the k1 = 0 plane, gaussian.f90:220-236
  if (tid < 3) {
    double* q = fr + 150 * tid;
    for (int k = 1; k <= 5; ++k) {
      int kk = (k == 1) ? 1 : 7 - k;
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
  __syncthreads();
  double* b1 = sb;
  double* b2 = sb + 150;
  double* b3 = sb + 300;
  double* a1 = sa;
  double* a2 = sa + 150;
  double* a3 = sa + 300;
  // OU update and solenoidal projection, gaussian.f90:243-274
  for (int m = tid; m < 150; m += blockDim.x) {
    int i = 1 + m % 6, j = 1 + (m / 6) % 5, k = 1 + m / 30;
    double kx = kxr6[i - 1], ky = kyr5[j - 1], kz = kzr5[k - 1];
    double radm = sqrt(kx * kx + ky * ky + kz * kz);
    if (radm < xkf) {
      b1[m] = b1[m] * (1.0 - dt / tf) + fr[m];
      b2[m] = b2[m] * (1.0 - dt / tf) + fr[m + 150];
      b3[m] = b3[m] * (1.0 - dt / tf) + fr[m + 300];
      double t1 = kx * b1[m], t2 = ky * b2[m], t3 = kz * b3[m];
      double rs = radm + smallx;
      double divb = (t1 + t2 + t3) / (rs * rs);
      if (radm == 0.0) divb = 0.0;
      a1[m] = b1[m] - kx * divb;
      a2[m] = b2[m] - ky * divb;
      a3[m] = b3[m] - kz * divb;
    } else {
      a1[m] = 0.0; a2[m] = 0.0; a3[m] = 0.0;
    }
  }
  __syncthreads();
  // gaussian.f90:277-307
  if (tid < 3) {
    double* a = sa + 150 * tid;
    a[m655(1, 1, 1)] = 0.0;
    a[m655(2, 1, 1)] = 0.0;
    for (int k = 1; k <= 5; ++k) {
      int kk = (k == 1) ? 1 : 7 - k;
      for (int j = 2; j <= 3; ++j) {
        int jj = 7 - j;
        a[m655(1, jj, kk)] = a[m655(1, j, k)];
        a[m655(2, jj, kk)] = -a[m655(2, j, k)];
      }
    }
    for (int k = 2; k <= 3; ++k) {
      int kk = 7 - k;
      a[m655(1, 1, kk)] = a[m655(1, 1, k)];
      a[m655(2, 1, kk)] = -a[m655(2, 1, k)];
    }
  }
  __syncthreads();
  for (int m = tid; m < 450; m += blockDim.x) {
    st->b[m] = sb[m];
    st->a[m] = sa[m];
  }
  if (tid < 32) st->ivf[tid] = siv[tid];
  if (tid == 0) {
    st->iseedf = sstate[0];
    st->iyf = sstate[1];
  }
}
__global__ void __launch_bounds__(256) k_forcing_update(ForcingDev* st, double var, double tf,
                                                        double pi2, const double* kxr6,
                                                        const double* kyr5, const double* kzr5) {
  k_forcing_update_body(blockIdx.x, gridDim.x, st, var, tf, pi2, kxr6, kyr5, kzr5);
}

}  // namespace

namespace {
// one block per box: keep the state, then the update
__global__ void __launch_bounds__(256) k_forcing_update_multi(const BoxForcing* boxes) {
  const BoxForcing& B = boxes[blockIdx.y];
  const int n = (int)(sizeof(ForcingDev) / sizeof(int32_t));
  const int32_t* src = reinterpret_cast<const int32_t*>(B.st);
  int32_t* dst = reinterpret_cast<int32_t*>(B.backup);
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  k_forcing_update_body(0, 1, B.st, B.var, B.tf, B.pi2, B.kxr6, B.kyr5, B.kzr5);
}
}  // namespace

void launch_forcing_update_multi(const BoxForcing* boxes, int nb, cudaStream_t s) {
  if (nb <= 0) return;
  k_forcing_update_multi<<<dim3(1, nb), 256, 0, s>>>(boxes);
  count_launch();
}

void launch_forcing_update(ForcingDev* st, double var, double tf, double pi2,
                           const double* kxr6, const double* kyr5, const double* kzr5,
                           cudaStream_t s) {
  { k_forcing_update<<<1, 256, 0, s>>>(st, var, tf, pi2, kxr6, kyr5, kzr5); count_launch(); }
}

}  // namespace lbm
