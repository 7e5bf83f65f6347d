// lbm_staged.cu - the fused stream + collide step with its input rows staged
// through shared memory by the bulk-copy (TMA) engine.
//
// Same arithmetic and the same result as k_fused (lbm_fluid.cu): per node the
// 19 post-streaming populations are read, collided with collision_MRT's MRT
// operator and Guo forcing (B/collision.f90:31-208) and pushed to their
// neighbours (the cshift streaming of B/streaming.f90:13-166), bouncing back
// at the x walls of the channel (C/streaming.f90:175-187).  What changes is
// how the loads move.  A persistent CTA owns a contiguous run of x-rows (one
// row = the nx nodes of one (y, z)) and is warp-specialised:
//
//   producer  warp 0 keeps S rows in flight: per row, lanes 0..18 each issue
//             the cp.async.bulk copy global -> shared of one population row
//             and lane 19 the flag row, all completing on the stage's "full"
//             mbarrier (transaction count = bytes of the row);
//   consumers the other warps wait for a stage, collide its nodes from shared
//             memory, store the pushed populations straight to HBM (each warp
//             writes 32 consecutive values per direction), and release the
//             stage on its "empty" mbarrier.
//
// The loads are whole, 16-byte aligned rows that never wait on a thread's
// registers: the number of bytes in flight is set by S, not by how many
// warps the collision's register count lets an SM hold.  Requires nx a
// multiple of 4 (row copies are multiples of 16 bytes).
//
// Every wait on an mbarrier is bounded: after kWaitNs the kernel records
// LBM_ERR_TIMEOUT in DevStatus, lets the copies it issued land and returns.
#include "lbm_internal.cuh"
#include "lbm_collide.cuh"
#include "lbm_f32x2.cuh"
#include "lbm_pipeline.cuh"

namespace lbm {

namespace {

// Shared memory of one CTA: S input stages, each holding the 19 population
// rows, the solid-mask row and the force-series coefficients of the row for the
// two force fields (kRowCoef values each); then the full and empty mbarriers
// of every stage and an abort flag.
template <typename T>
struct StagedLayout {
  int nx, S, sw;
  __host__ __device__ size_t coef_offset() const {
    return (size_t)nx * NPOP * sizeof(T) + (size_t)sw * 4;
  }
  __host__ __device__ size_t stage_bytes() const { return coef_offset() + 2 * kRowCoef * sizeof(T); }
  __host__ __device__ size_t bar_offset() const { return S * stage_bytes(); }
  __host__ __device__ size_t total() const { return bar_offset() + 16 * (size_t)S + 16; }
};

// Producer warp: keeps the CTA's rows flowing into the S stages.  Lane q < 19
// copies population row q, lane 19 the solid-mask row, lanes 20 and 21 the force
// coefficients of the row (tabulated forcing only).
template <typename T>
__device__ void stage_producer(const StagedLayout<T>& L, unsigned char* smem, uint64_t* full,
                               uint64_t* empty, volatile int* abort_flag, int row0, int nloc,
                               const T* __restrict__ fin, const uint32_t* __restrict__ mask,
                               const ForceView<T>& fa, const ForceView<T>& fb, int N,
                               DevStatus* st) {
  const int lane = threadIdx.x & 31, S = L.S, nx = L.nx;
  const unsigned row_bytes = (unsigned)(nx * sizeof(T));
  const bool ta = fa.mode == FM_TABLE, tb = fb.mode == FM_TABLE;
  const unsigned coef_bytes = kRowCoef * sizeof(T);
  const unsigned tx = (unsigned)L.coef_offset() + (ta ? coef_bytes : 0) + (tb ? coef_bytes : 0);
  int issued = 0;
  for (int j = 0; j < nloc; ++j) {
    const int s = j % S;
    bool ok = true;
    if (j >= S) ok = mbar_wait_bounded(empty + s, (unsigned)(((j / S) - 1) & 1), kWaitNs);
    if (__any_sync(0xffffffffu, !ok) || *abort_flag) {
      if (lane == 0 && !*abort_flag) {
        *abort_flag = 1;
        raise_error(st, LBM_ERR_TIMEOUT, blockIdx.x);
      }
      break;
    }
    unsigned char* stage = smem + (size_t)s * L.stage_bytes();
    T* dst = reinterpret_cast<T*>(stage);
    const int row = row0 + j;
    const size_t base = (size_t)row * nx;
    if (lane == 0) mbar_arrive_expect_tx(full + s, tx);
    __syncwarp();
    if (lane < NPOP)
      bulk_g2s(dst + (size_t)lane * nx, fin + (size_t)lane * N + base, row_bytes, full + s);
    else if (lane == NPOP)
      bulk_g2s(dst + (size_t)NPOP * nx, mask + (size_t)row * L.sw, (unsigned)(L.sw * 4), full + s);
    else if (lane == NPOP + 1 && ta)
      bulk_g2s(stage + L.coef_offset(), fa.rowtab + (size_t)row * kRowCoef, coef_bytes, full + s);
    else if (lane == NPOP + 2 && tb)
      bulk_g2s(stage + L.coef_offset() + coef_bytes, fb.rowtab + (size_t)row * kRowCoef,
               coef_bytes, full + s);
    issued = j + 1;
  }
  // every copy issued must land before the CTA's shared memory goes away
  if (lane == 0)
    for (int j = issued > S ? issued - S : 0; j < issued; ++j)
      (void)mbar_wait_bounded(full + (j % S), (unsigned)((j / S) & 1), kWaitNs);
}

// Body force of one field at the x position with twiddles (c1, s1, c2, s2),
// the row's coefficients k in shared memory (tabulated forcing).
template <typename T>
__device__ __forceinline__ void row_force(const ForceView<T>& v, const T* k, T c1, T s1, T c2,
                                          T s2, T (&o)[3]) {
  if (v.mode == FM_TABLE) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      o[c] = k[5 * c] + k[5 * c + 1] * c1 + k[5 * c + 2] * s1 + k[5 * c + 3] * c2 + k[5 * c + 4] * s2;
  } else if (v.mode == FM_CONST) {
    o[0] = v.cfx; o[1] = v.cfy; o[2] = v.cfz;
  } else {
    o[0] = T(0); o[1] = T(0); o[2] = T(0);
  }
}

// Scalar consumers: one node per thread.  One producer warp (warp 0) and
// W = blockDim/32 - 1 consumer warps.
// FX (FP64 only): collide with exact fixed-point moment sums (collide_fx),
// falling back to collide_fast for the nodes it declines.
template <typename T, bool CHANNEL, bool FX = false>
__global__ void __launch_bounds__(288) k_fused_staged(Geometry g, RatesT<T> r,
                                                      const T* __restrict__ fin,
                                                      T* __restrict__ fout,
                                                      const int32_t* __restrict__ isnodes,
                                                      ForceView<T> fprev, ForceView<T> fnew,
                                                      int S, DevStatus* st) {
  extern __shared__ __align__(128) unsigned char smem[];
  const StagedLayout<T> L{g.nx, S, g.sw};
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int nrows = ny * nz;
  const int N = (int)g.N;
  const int nxy = nx * ny;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bar_offset());
  uint64_t* empty = full + S;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + S);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int W = (blockDim.x >> 5) - 1;

  // contiguous run of rows owned by this CTA
  const int row0 = (int)((long long)blockIdx.x * nrows / gridDim.x);
  const int nloc = (int)((long long)(blockIdx.x + 1) * nrows / gridDim.x) - row0;
  if (nloc <= 0) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, W);
    }
    *abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == 0) {
    stage_producer<T>(L, smem, full, empty, abort_flag, row0, nloc, fin, solid_mask(isnodes, g),
                      fprev, fnew, N, st);
    return;
  }

  // ---- consumers
  const int ct = threadIdx.x - 32;
  for (int i = 0; i < nloc; ++i) {
    const int s = i % S;
    const int row = row0 + i;
    const int z = row / ny, y = row - z * ny;
    const bool ok = mbar_wait_bounded(full + s, (unsigned)((i / S) & 1), kWaitNs);
    if (!ok || *abort_flag) {
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        raise_error(st, LBM_ERR_TIMEOUT, blockIdx.x);
      }
      break;
    }
    const unsigned char* stage = smem + (size_t)s * L.stage_bytes();
    const T* in = reinterpret_cast<const T*>(stage);
    const uint32_t* mrow = reinterpret_cast<const uint32_t*>(in + (size_t)NPOP * nx);
    const T* ka = reinterpret_cast<const T*>(stage + L.coef_offset());
    const T* kb = ka + kRowCoef;
    const int n0 = nxy * z + nx * y;
    const int oyp = (y == ny - 1) ? nx - nxy : nx, oym = (y == 0) ? nxy - nx : -nx;
    const int ozp = (z == nz - 1) ? nxy - N : nxy, ozm = (z == 0) ? N - nxy : -nxy;
    for (int x = ct; x < nx; x += 32 * W) {
      T f[NPOP];
#pragma unroll
      for (int q = 0; q < NPOP; ++q) f[q] = in[q * nx + x];
      if (!((mrow[x >> 5] >> (x & 31)) & 1u)) {
        const T c1 = fnew.xtw[4 * x], s1 = fnew.xtw[4 * x + 1];
        const T c2 = fnew.xtw[4 * x + 2], s2 = fnew.xtw[4 * x + 3];
        T fp[3], fc[3];
        row_force(fprev, ka, c1, s1, c2, s2, fp);
        row_force(fnew, kb, c1, s1, c2, s2, fc);
        bool done = false;
        if constexpr (FX) {
          done = collide_fx(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
          if (!done) {
#pragma unroll
            for (int q = 0; q < NPOP; ++q) f[q] = in[q * nx + x];
          }
        }
        if (!done) collide_fast(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
      }
      // 32-bit element indices: 19 N < 2^31 (N < 2^26 is enforced)
      const int n = n0 + x;
      const int oxp = (x == nx - 1) ? 1 - nx : 1, oxm = (x == 0) ? nx - 1 : -1;
#pragma unroll
      for (int q = 0; q < NPOP; ++q) {
        const int cx = cix(q), cy = ciy(q), cz = ciz(q);
        if (CHANNEL && ((cx == -1 && x == 0) || (cx == 1 && x == nx - 1))) {
          // halfway bounce-back at the wall (C/streaming.f90:175-187)
          fout[ipopp(q) * N + n] = f[q];
          continue;
        }
        const int off = (cx > 0 ? oxp : (cx < 0 ? oxm : 0)) + (cy > 0 ? oyp : (cy < 0 ? oym : 0)) +
                        (cz > 0 ? ozp : (cz < 0 ? ozm : 0));
        fout[q * N + n + off] = f[q];
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + s);   // this warp is done with stage s
  }
}

// Packed FP32 consumers: each thread owns the node pair (x0, x0 + 1), x0 even,
// and collides both with the f32x2 instructions.  The consumer warps form G
// groups of Wg = ceil(nx / 64) warps; group k takes the CTA's rows k, k + G,
// ... so that several rows are in the collision at once.
template <bool CHANNEL>
__global__ void __launch_bounds__(288) k_fused_staged_x2(Geometry g, RatesT<F2> r,
                                                         const float* __restrict__ fin,
                                                         float* __restrict__ fout,
                                                         const int32_t* __restrict__ isnodes,
                                                         ForceView<float> fprev,
                                                         ForceView<float> fnew, int S,
                                                         DevStatus* st) {
  extern __shared__ __align__(128) unsigned char smem[];
  const StagedLayout<float> L{g.nx, S, g.sw};
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int nrows = ny * nz;
  const int N = (int)g.N;
  const int nxy = nx * ny;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bar_offset());
  uint64_t* empty = full + S;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + S);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Wg = (nx + 63) / 64;
  const int G = ((blockDim.x >> 5) - 1) / Wg;
  // Row i goes to group i % G and stage i % S.  With S a multiple of G each
  // stage belongs to one group, which waits for use u of a stage only after
  // consuming use u - 1 itself; otherwise a wait on parity u & 1 could be
  // satisfied by use u - 2.  The host plans only such schedules.
  if (G < 1 || S % G != 0) {
    if (threadIdx.x == 0) raise_error(st, LBM_ERR_ARG, blockIdx.x);
    return;
  }

  const int row0 = (int)((long long)blockIdx.x * nrows / gridDim.x);
  const int nloc = (int)((long long)(blockIdx.x + 1) * nrows / gridDim.x) - row0;
  if (nloc <= 0) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, Wg);
    }
    *abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == 0) {
    stage_producer<float>(L, smem, full, empty, abort_flag, row0, nloc, fin,
                          solid_mask(isnodes, g), fprev, fnew, N, st);
    return;
  }
  const int cw = warp - 1;
  const int grp = cw / Wg;
  if (grp >= G) return;  // (blockDim is sized so this does not happen)
  const int x0 = 2 * ((cw - grp * Wg) * 32 + lane);
  const bool active = x0 < nx;
  // x twiddles of the pair, the same for every row
  F2 c1 = F2(0.0), s1 = F2(0.0), c2 = F2(0.0), s2 = F2(0.0);
  if (active) {
    const float* t = fnew.xtw + 4 * x0;
    c1 = pack2(t[0], t[4]); s1 = pack2(t[1], t[5]);
    c2 = pack2(t[2], t[6]); s2 = pack2(t[3], t[7]);
  }
  auto force2 = [&](const ForceView<float>& v, const float* k, F2 (&o)[3]) {
    if (v.mode == FM_TABLE) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        o[c] = splat2(k[5 * c]) + splat2(k[5 * c + 1]) * c1 + splat2(k[5 * c + 2]) * s1 +
               splat2(k[5 * c + 3]) * c2 + splat2(k[5 * c + 4]) * s2;
    } else if (v.mode == FM_CONST) {
      o[0] = splat2(v.cfx); o[1] = splat2(v.cfy); o[2] = splat2(v.cfz);
    } else {
      o[0] = F2(0.0); o[1] = F2(0.0); o[2] = F2(0.0);
    }
  };

  for (int i = grp; i < nloc; i += G) {
    const int s = i % S;
    const int row = row0 + i;
    const int z = row / ny, y = row - z * ny;
    const bool ok = mbar_wait_bounded(full + s, (unsigned)((i / S) & 1), kWaitNs);
    if (!ok || *abort_flag) {
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        raise_error(st, LBM_ERR_TIMEOUT, blockIdx.x);
      }
      break;
    }
    const unsigned char* stage = smem + (size_t)s * L.stage_bytes();
    const float* in = reinterpret_cast<const float*>(stage);
    if (active) {
      const uint32_t mw = reinterpret_cast<const uint32_t*>(in + (size_t)NPOP * nx)[x0 >> 5];
      F2 f[NPOP];
#pragma unroll
      for (int q = 0; q < NPOP; ++q)
        f[q] = F2(*reinterpret_cast<const unsigned long long*>(in + q * nx + x0), 0);
      const bool fl0 = !((mw >> (x0 & 31)) & 1u), fl1 = !((mw >> ((x0 + 1) & 31)) & 1u);
      if (fl0 || fl1) {
        const float* ka = reinterpret_cast<const float*>(stage + L.coef_offset());
        F2 fp[3], fc[3];
        force2(fprev, ka, fp);
        force2(fnew, ka + kRowCoef, fc);
        collide_fast(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
        if (!(fl0 && fl1)) {
          // one node of the pair is solid: it keeps its populations
#pragma unroll
          for (int q = 0; q < NPOP; ++q) {
            float lo, hi;
            unpack2(f[q], lo, hi);
            if (fl0) hi = in[q * nx + x0 + 1];
            else lo = in[q * nx + x0];
            f[q] = pack2(lo, hi);
          }
        }
      }
      // push; 32-bit element indices (19 N < 2^31)
      const int n = nxy * z + nx * y + x0;
      const int oyp = (y == ny - 1) ? nx - nxy : nx, oym = (y == 0) ? nxy - nx : -nx;
      const int ozp = (z == nz - 1) ? nxy - N : nxy, ozm = (z == 0) ? N - nxy : -nxy;
      const bool left = x0 == 0, right = x0 + 2 == nx;
#pragma unroll
      for (int q = 0; q < NPOP; ++q) {
        const int cx = cix(q), cy = ciy(q), cz = ciz(q);
        const int idx = q * N + n + (cy > 0 ? oyp : (cy < 0 ? oym : 0)) +
                        (cz > 0 ? ozp : (cz < 0 ? ozm : 0));
        if (cx == 0) {
          *reinterpret_cast<unsigned long long*>(fout + idx) = f[q].v;
          continue;
        }
        float lo, hi;
        unpack2(f[q], lo, hi);
        if (cx > 0) {
          fout[idx + 1] = lo;
          if (!right) fout[idx + 2] = hi;
          else if (CHANNEL) fout[ipopp(q) * N + n + 1] = hi;  // wall at x = nx - 1/2
          else fout[idx + 2 - nx] = hi;
        } else {
          fout[idx] = hi;
          if (!left) fout[idx - 1] = lo;
          else if (CHANNEL) fout[ipopp(q) * N + n] = lo;  // wall at x = -1/2
          else fout[idx - 1 + nx] = lo;
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + s);   // this warp is done with stage s
  }
}

}  // namespace

// ---------------------------------------------------------------------------
template <typename T>
bool staged_eligible(const Geometry& g, int S, bool packed) {
  if (g.nx % 4 != 0 || S < 2) return false;
  if (packed && (sizeof(T) != 4 || g.nx > 512)) return false;
  const StagedLayout<T> L{g.nx, S, g.sw};
  return L.total() <= 227 * 1024;
}

template <typename T>
int staged_max_stages(const Geometry& g) {
  int best = 0;
  for (int S = 2; S <= 8; ++S)
    if (staged_eligible<T>(g, S, false)) best = S;
  return best;
}

template <typename T>
static void* staged_kernel(bool channel, bool packed, bool fx) {
  if (packed) {
    if constexpr (sizeof(T) == 4)
      return channel ? (void*)k_fused_staged_x2<true> : (void*)k_fused_staged_x2<false>;
    return nullptr;
  }
  if constexpr (sizeof(T) == 8) {
    if (fx) return channel ? (void*)k_fused_staged<T, true, true> : (void*)k_fused_staged<T, false, true>;
  }
  return channel ? (void*)k_fused_staged<T, true> : (void*)k_fused_staged<T, false>;
}

// Plan a launch of the staged kernel (packed: the FP32 pair kernel) with S
// stages and ctas_per_sm CTAs resident per SM (0: as many as fit).  Returns
// false when the plan does not apply.
template <typename T>
bool plan_fused_staged(const Geometry& g, int S, int ctas_per_sm, bool packed, int groups,
                       StagedPlan* plan, bool fx) {
  fx = fx && sizeof(T) == 8 && !packed;
  if (!staged_eligible<T>(g, S, packed)) return false;
  const StagedLayout<T> L{g.nx, S, g.sw};
  int dev = 0, sms = 0, fit = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  const void* kern = staged_kernel<T>(g.channel != 0, packed, fx);
  if (!kern) return false;
  // the largest plan any caller may launch, so plans can alternate freely
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
      cudaSuccess)
    return false;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int consumers;
  if (packed) {
    const int wg = (g.nx + 63) / 64;
    const int gmax = 8 / wg;
    // every stage must always be consumed by the same group (S a multiple of
    // G): a group then waits on a stage only after it consumed the stage's
    // previous use itself, so the phase parity it waits for is unambiguous
    if (groups < 1 || groups > gmax || S % groups != 0) return false;
    consumers = wg * groups;
  } else {
    if (groups != 1) return false;
    consumers = g.nx >= 256 ? 8 : (g.nx + 31) / 32;
  }
  plan->threads = 32 * (consumers + 1);
  plan->smem = L.total();
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, plan->threads, plan->smem) !=
          cudaSuccess ||
      fit < 1)
    return false;
  const int per_sm = ctas_per_sm > 0 ? (ctas_per_sm < fit ? ctas_per_sm : fit) : fit;
  const int nrows = g.ny * g.nz;
  plan->S = S;
  plan->packed = packed;
  plan->groups = groups;
  plan->fx = fx;
  plan->ctas_per_sm = per_sm;
  plan->grid = nrows < sms * per_sm ? nrows : sms * per_sm;
  return true;
}

template <typename T>
void launch_fused_staged(const Geometry& g, const Rates& r, const T* fin, T* fout,
                         const int32_t* isnodes, const ForceView<T>& fprev,
                         const ForceView<T>& fnew, const StagedPlan& p, DevStatus* st,
                         cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (p.packed) {
      const RatesT<F2> r2 = rates_t<F2>(r);
      if (g.channel)
        k_fused_staged_x2<true><<<p.grid, p.threads, p.smem, s>>>(g, r2, fin, fout, isnodes, fprev,
                                                                  fnew, p.S, st);
      else
        k_fused_staged_x2<false><<<p.grid, p.threads, p.smem, s>>>(g, r2, fin, fout, isnodes,
                                                                   fprev, fnew, p.S, st);
      count_launch();
      return;
    }
  }
  if constexpr (sizeof(T) == 8) {
    if (p.fx) {
      if (g.channel)
        k_fused_staged<T, true, true><<<p.grid, p.threads, p.smem, s>>>(
            g, rates_t<T>(r), fin, fout, isnodes, fprev, fnew, p.S, st);
      else
        k_fused_staged<T, false, true><<<p.grid, p.threads, p.smem, s>>>(
            g, rates_t<T>(r), fin, fout, isnodes, fprev, fnew, p.S, st);
      count_launch();
      return;
    }
  }
  if (g.channel)
    k_fused_staged<T, true><<<p.grid, p.threads, p.smem, s>>>(g, rates_t<T>(r), fin, fout, isnodes,
                                                              fprev, fnew, p.S, st);
  else
    k_fused_staged<T, false><<<p.grid, p.threads, p.smem, s>>>(g, rates_t<T>(r), fin, fout,
                                                               isnodes, fprev, fnew, p.S, st);
  count_launch();
}

#define LBM_STAGED_INSTANTIATE(T)                                                            \
  template bool staged_eligible<T>(const Geometry&, int, bool);                              \
  template int staged_max_stages<T>(const Geometry&);                                        \
  template bool plan_fused_staged<T>(const Geometry&, int, int, bool, int, StagedPlan*, bool); \
  template void launch_fused_staged<T>(const Geometry&, const Rates&, const T*, T*,          \
                                       const int32_t*, const ForceView<T>&,                  \
                                       const ForceView<T>&, const StagedPlan&, DevStatus*,   \
                                       cudaStream_t);
LBM_STAGED_INSTANTIATE(float)
LBM_STAGED_INSTANTIATE(double)

}  // namespace lbm
