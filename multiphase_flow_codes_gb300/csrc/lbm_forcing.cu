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

// One block: thread 0 draws the 450 uniform numbers in the reference's
// order (mc, k, j, i = 1,3,5; cont1 then rph), then the magnitudes,
// phases, Ornstein-Uhlenbeck update and projection run one mode per thread.
__device__ __forceinline__ void k_forcing_update_body(int bx, int gx, ForcingDev* st, double var, double tf,
                                                        double pi2, const double* kxr6,
                                                        const double* kyr5, const double* kzr5) {
  __shared__ double u[450];
  __shared__ double fr[450];
  const int tid = threadIdx.x;
  const double smallx = 1.0e-18;
  const double xkf = sqrt(8.0);
  const double dt = 1.0;
  if (tid == 0) {
    int32_t idum = st->iseedf, iy = st->iyf;
    int32_t iv[32];
    for (int i = 0; i < 32; ++i) iv[i] = st->ivf[i];
    for (int d = 0; d < 450; ++d) u[d] = ran1_dev(&idum, &iy, iv);
    st->iseedf = idum;
    st->iyf = iy;
    for (int i = 0; i < 32; ++i) st->ivf[i] = iv[i];
  }
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
  double* b1 = st->b;
  double* b2 = st->b + 150;
  double* b3 = st->b + 300;
  double* a1 = st->a;
  double* a2 = st->a + 150;
  double* a3 = st->a + 300;
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
    double* a = st->a + 150 * tid;
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
