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
#include <mutex>

#include "lbm_internal.cuh"

namespace {

constexpr int kMaxDevices = 64;

// per-plane partial sums (mass, momentum x, y, z) of the last call
__device__ __align__(256) double g_plane_sums[LBM_NOALLOC_MAX_PLANES * 4];

// device address of g_plane_sums, looked up once per device
double* g_plane_sums_addr[kMaxDevices] = {nullptr};
std::mutex g_addr_mutex;

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

// Device address of the scratch array on the current device, looked up
// (cudaGetSymbolAddress) on the first call made with that device current.
cudaError_t scratch_on_current_device(double** ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (g_plane_sums_addr[dev] == nullptr) {
    double* p = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_plane_sums);
    if (e != cudaSuccess) return e;
    g_plane_sums_addr[dev] = p;
  }
  *ptr = g_plane_sums_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int lbm_mass_momentum_noalloc(const double* f, int nx, int ny, int nz, double* out,
                                         void* stream) {
  if (!f || !out || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_ARG;
  if (nz > LBM_NOALLOC_MAX_PLANES) return LBM_ERR_ARG;  // scratch holds one sum per plane
  if ((long long)nx * ny > (1LL << 30)) return LBM_ERR_ARG;
  double* sums = nullptr;
  if (scratch_on_current_device(&sums) != cudaSuccess) return LBM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long N = (long long)nx * ny * nz;
  k_plane_sums<<<nz, 256, 0, s>>>(f, nx, ny, N, sums);
  lbm::count_launch();
  k_plane_total<<<1, 256, 0, s>>>(sums, nz, out);
  lbm::count_launch();
  return cudaGetLastError() == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}
