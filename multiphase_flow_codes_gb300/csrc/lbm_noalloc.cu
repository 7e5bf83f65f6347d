// lbm_noalloc.cu - mass and momentum totals of a caller-held population
// field, computed without allocating any memory.
//
// Some callers of this library cannot call cudaMalloc: a host solver that
// has already reserved the GPU's memory for its own state and forbids any
// further allocation, or an embedding runtime that owns all device memory
// through its own pool and only hands out pointers to it.  For them
// lbm_mass_momentum_noalloc works with the caller's input and output buffers
// alone.  Its scratch space (one partial sum per z-plane) is the file-scope
// device array below: every GPU that loads this library holds it (128 KiB)
// until the process exits, and every call shares it.
#include "lbm_internal.cuh"

namespace {

// per-plane partial sums (mass, momentum x, y, z) of the last call
__device__ __align__(256) double g_plane_sums[LBM_NOALLOC_MAX_PLANES * 4];

// Stage 1: block z sums plane z into g_plane_sums (every entry the second
// stage reads is written first, so no clearing is needed).  Deterministic:
// fixed per-thread order, fixed tree.
__global__ void __launch_bounds__(256) k_plane_sums(const double* __restrict__ f, int nx, int ny,
                                                    long long N, double* __restrict__ sums) {
  const int z = blockIdx.x;
  const long long base = (long long)z * nx * ny;
  const int plane = nx * ny;
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  for (int t = threadIdx.x; t < plane; t += blockDim.x) {
    const long long n = base + t;
#pragma unroll
    for (int q = 0; q < lbm::NPOP; ++q) {
      const double v = f[(long long)q * N + n];
      m[0] += v;
      m[1] += lbm::cix(q) * v;
      m[2] += lbm::ciy(q) * v;
      m[3] += lbm::ciz(q) * v;
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
  if (threadIdx.x < 4) sums[4 * z + threadIdx.x] = sm[threadIdx.x][0];
}

// Stage 2: one block adds the plane sums in plane order into out[0..3].
__global__ void __launch_bounds__(256) k_plane_total(const double* __restrict__ sums, int nz,
                                                     double* __restrict__ out) {
  __shared__ double sm[4][256];
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  for (int z = threadIdx.x; z < nz; z += blockDim.x)
    for (int c = 0; c < 4; ++c) m[c] += sums[4 * z + c];
  for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] = m[c];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sm[threadIdx.x][0];
}

// Device address of the scratch array in the current context.  It is looked
// up on every call (cudaGetSymbolAddress allocates nothing): a cached value
// would go stale for a caller that runs its own driver-API context or
// recreates the context after cudaDeviceReset, since each context holds its
// own instance of the array.
cudaError_t scratch_in_current_context(double** ptr) {
  double* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_plane_sums);
  if (e != cudaSuccess) return e;
  *ptr = p;
  return cudaSuccess;
}

}  // namespace

extern "C" int lbm_mass_momentum_noalloc(const double* f, int nx, int ny, int nz, double* out,
                                         void* stream) {
  if (!f || !out || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_ARG;
  if (nz > LBM_NOALLOC_MAX_PLANES) return LBM_ERR_ARG;  // scratch holds one sum per plane
  if ((long long)nx * ny > (1LL << 30)) return LBM_ERR_ARG;
  // An error left pending by earlier work is not this call's: report it as
  // such, launch nothing and leave it for its owner to read.
  if (cudaPeekAtLastError() != cudaSuccess) return LBM_ERR_STATE;
  double* sums = nullptr;
  if (scratch_in_current_context(&sums) != cudaSuccess) return LBM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long N = (long long)nx * ny * nz;
  k_plane_sums<<<nz, 256, 0, s>>>(f, nx, ny, N, sums);
  lbm::count_launch();
  if (cudaGetLastError() != cudaSuccess) return LBM_ERR_CUDA;  // this launch's own error
  k_plane_total<<<1, 256, 0, s>>>(sums, nz, out);
  lbm::count_launch();
  if (cudaGetLastError() != cudaSuccess) return LBM_ERR_CUDA;
  return LBM_OK;
}
