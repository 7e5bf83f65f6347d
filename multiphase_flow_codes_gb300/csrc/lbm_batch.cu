// lbm_batch.cu - one persistent kernel that streams and collides many
// independent boxes of different sizes in FP32 (populations as deviations
// f_i - w_i rho0).
//
// The work is a list of tasks; a task is up to kTaskNodes nodes of one box:
// k consecutive x-rows of one z-plane (k rows of nx nodes are contiguous in
// every population array, so each population of a task is one bulk copy).
// Each CTA owns a contiguous run of tasks and runs the producer / consumer
// pipeline of k_fused_staged_x2 (lbm_staged.cu) over them: warp 0 streams
// the task's 19 population segments, its solid-mask rows and its force
// coefficient rows into a shared-memory stage; consumer warps (groups of two,
// one node pair per thread) collide the nodes with the f32x2 arithmetic and
// push them within their own box (periodic, or bounced back at the box's x
// walls in the channel form).  Per-node arithmetic is the single-box
// kernel's, so a box gives the same result in a batch of any composition.
#include "lbm_internal.cuh"
#include "lbm_collide.cuh"
#include "lbm_f32x2.cuh"
#include "lbm_pipeline.cuh"

namespace lbm {

namespace {

constexpr int kTaskNodes = 128;
constexpr int kMaskWords = 4 * (kTaskNodes / 32);  // mask words of the rows of one task (<= 16)

// stage: 19 population segments of kTaskNodes, mask words, two coefficient
// blocks of up to kTaskNodes/32*... rows (at most 4 rows of kRowCoef)
constexpr int kMaxTaskRows = kTaskNodes / 32;
constexpr size_t kPopBytes = (size_t)NPOP * kTaskNodes * sizeof(float);
constexpr size_t kMaskOff = kPopBytes;
constexpr size_t kCoefOff = kMaskOff + kMaskWords * 4;
constexpr size_t kCoefBytes = (size_t)kMaxTaskRows * kRowCoef * sizeof(float);
constexpr size_t kStageBytes = kCoefOff + 2 * kCoefBytes;
static_assert(kStageBytes % 16 == 0, "stage must keep 16-byte alignment");

__host__ __device__ inline size_t batch_smem(int S) { return S * kStageBytes + 16 * (size_t)S + 16; }

template <bool CHANNEL>
__global__ void __launch_bounds__(288) k_fused_batch_x2(const BatchBox* __restrict__ boxes,
                                                        const BatchTask* __restrict__ tasks,
                                                        int ntasks, BatchPhase ph, RatesT<F2> r,
                                                        int S, DevStatus* st) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * kStageBytes);
  uint64_t* empty = full + S;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + S);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int Wg = kTaskNodes / 64;
  const int G = ((blockDim.x >> 5) - 1) / Wg;
  // task i goes to group i % G and stage i % S; S a multiple of G keeps every
  // stage with one group (see k_fused_staged_x2)
  if (G < 1 || S % G != 0) {
    if (threadIdx.x == 0) raise_error(st, LBM_ERR_ARG, blockIdx.x);
    return;
  }
  const int t0 = (int)((long long)blockIdx.x * ntasks / gridDim.x);
  const int nloc = (int)((long long)(blockIdx.x + 1) * ntasks / gridDim.x) - t0;
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
    // ---- producer
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
      const BatchTask tk = tasks[t0 + j];
      const BatchBox& b = boxes[tk.box];
      const int nodes = tk.nrows * b.nx;
      const size_t base = (size_t)tk.row0 * b.nx;
      const bool ta = ph.prev_mode == FM_TABLE, tb = ph.new_mode == FM_TABLE;
      const unsigned coef = (unsigned)(tk.nrows * kRowCoef * sizeof(float));
      const unsigned tx = (unsigned)(NPOP * nodes * sizeof(float) + tk.nrows * b.sw * 4) +
                          (ta ? coef : 0) + (tb ? coef : 0);
      unsigned char* stage = smem + (size_t)s * kStageBytes;
      if (lane == 0) mbar_arrive_expect_tx(full + s, tx);
      __syncwarp();
      const float* fin = b.f[ph.cur];
      if (lane < NPOP) {
        bulk_g2s(stage + (size_t)lane * kTaskNodes * sizeof(float), fin + (size_t)lane * b.N + base,
                 (unsigned)(nodes * sizeof(float)), full + s);
      } else if (lane == NPOP) {
        const uint32_t* mask = solid_mask_raw(b.flags[ph.fcur], b.N);
        bulk_g2s(stage + kMaskOff, mask + (size_t)tk.row0 * b.sw, (unsigned)(tk.nrows * b.sw * 4),
                 full + s);
      } else if (lane == NPOP + 1 && ta) {
        bulk_g2s(stage + kCoefOff, b.rowtab[ph.prev_slot] + (size_t)tk.row0 * kRowCoef, coef,
                 full + s);
      } else if (lane == NPOP + 2 && tb) {
        bulk_g2s(stage + kCoefOff + kCoefBytes, b.rowtab[ph.new_slot] + (size_t)tk.row0 * kRowCoef,
                 coef, full + s);
      }
      issued = j + 1;
    }
    if (lane == 0)
      for (int j = issued > S ? issued - S : 0; j < issued; ++j)
        (void)mbar_wait_bounded(full + (j % S), (unsigned)((j / S) & 1), kWaitNs);
    return;
  }

  // ---- consumers: group grp, pair gt of the task
  const int cw = warp - 1;
  const int grp = cw / Wg;
  if (grp >= G) return;
  const int gt = (cw - grp * Wg) * 32 + lane;
  for (int i = grp; i < nloc; i += G) {
    const int s = i % S;
    const bool ok = mbar_wait_bounded(full + s, (unsigned)((i / S) & 1), kWaitNs);
    if (!ok || *abort_flag) {
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        raise_error(st, LBM_ERR_TIMEOUT, blockIdx.x);
      }
      break;
    }
    const BatchTask tk = tasks[t0 + i];
    const BatchBox& b = boxes[tk.box];
    const int nx = b.nx, ny = b.ny, nz = b.nz, N = b.N, nxy = nx * ny;
    const int t = 2 * gt;  // first node of the pair within the task
    if (t < tk.nrows * nx) {
      const unsigned char* stage = smem + (size_t)s * kStageBytes;
      const float* in = reinterpret_cast<const float*>(stage);
      const int rr = t / nx, x0 = t - rr * nx;
      const int row = tk.row0 + rr;
      const int z = row / ny, y = row - z * ny;
      const uint32_t mw = reinterpret_cast<const uint32_t*>(stage + kMaskOff)[rr * b.sw + (x0 >> 5)];
      F2 f[NPOP];
#pragma unroll
      for (int q = 0; q < NPOP; ++q)
        f[q] = F2(*reinterpret_cast<const unsigned long long*>(in + q * kTaskNodes + t), 0);
      const bool fl0 = !((mw >> (x0 & 31)) & 1u), fl1 = !((mw >> ((x0 + 1) & 31)) & 1u);
      if (fl0 || fl1) {
        const float* tw = b.xtw + 4 * x0;
        const F2 c1 = pack2(tw[0], tw[4]), s1 = pack2(tw[1], tw[5]);
        const F2 c2 = pack2(tw[2], tw[6]), s2 = pack2(tw[3], tw[7]);
        auto force2 = [&](int mode, const float* k, F2 (&o)[3]) {
          if (mode == FM_TABLE) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
              o[c] = splat2(k[5 * c]) + splat2(k[5 * c + 1]) * c1 + splat2(k[5 * c + 2]) * s1 +
                     splat2(k[5 * c + 3]) * c2 + splat2(k[5 * c + 4]) * s2;
          } else if (mode == FM_CONST) {
            o[0] = splat2(b.cfx); o[1] = splat2(b.cfy); o[2] = splat2(b.cfz);
          } else {
            o[0] = F2(0.0); o[1] = F2(0.0); o[2] = F2(0.0);
          }
        };
        const float* ka = reinterpret_cast<const float*>(stage + kCoefOff) + rr * kRowCoef;
        const float* kb = reinterpret_cast<const float*>(stage + kCoefOff + kCoefBytes) + rr * kRowCoef;
        F2 fp[3], fc[3];
        force2(ph.prev_mode, ka, fp);
        force2(ph.new_mode, kb, fc);
        collide_fast(f, fp[0], fp[1], fp[2], fc[0], fc[1], fc[2], r);
        if (!(fl0 && fl1)) {
#pragma unroll
          for (int q = 0; q < NPOP; ++q) {
            float lo, hi;
            unpack2(f[q], lo, hi);
            if (fl0) hi = in[q * kTaskNodes + t + 1];
            else lo = in[q * kTaskNodes + t];
            f[q] = pack2(lo, hi);
          }
        }
      }
      float* fout = b.f[1 - ph.cur];
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
          else if (CHANNEL) fout[ipopp(q) * N + n + 1] = hi;
          else fout[idx + 2 - nx] = hi;
        } else {
          fout[idx] = hi;
          if (!left) fout[idx - 1] = lo;
          else if (CHANNEL) fout[ipopp(q) * N + n] = lo;
          else fout[idx - 1 + nx] = lo;
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + s);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
int batch_task_rows(int nx, int ny) {
  int k = kTaskNodes / nx;
  if (k < 1) return 0;
  if (k > kMaxTaskRows) k = kMaxTaskRows;
  while (k > 1 && ny % k != 0) --k;
  return k;
}

bool batch_box_ok(const Geometry& g) {
  return g.nx % 4 == 0 && g.nx <= kTaskNodes && g.sw * batch_task_rows(g.nx, g.ny) <= kMaskWords;
}

bool plan_batch(bool channel, int S, int groups, int ctas_per_sm, int ntasks, StagedPlan* plan) {
  constexpr int Wg = kTaskNodes / 64;
  if (S < 2 || S > 8 || groups < 1 || groups * Wg > 8 || S % groups != 0) return false;
  const size_t smem = batch_smem(S);
  if (smem > 227 * 1024) return false;
  const void* kern = channel ? (const void*)k_fused_batch_x2<true> : (const void*)k_fused_batch_x2<false>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
      cudaSuccess)
    return false;
  int dev = 0, sms = 0, fit = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  plan->threads = 32 * (1 + groups * Wg);
  plan->smem = smem;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, plan->threads, plan->smem) !=
          cudaSuccess ||
      fit < 1)
    return false;
  const int per_sm = ctas_per_sm > 0 ? (ctas_per_sm < fit ? ctas_per_sm : fit) : fit;
  plan->S = S;
  plan->packed = true;
  plan->groups = groups;
  plan->ctas_per_sm = per_sm;
  plan->grid = ntasks < sms * per_sm ? ntasks : sms * per_sm;
  return plan->grid > 0;
}

void launch_fused_batch(bool channel, const BatchBox* boxes, const BatchTask* tasks, int ntasks,
                        const BatchPhase& ph, const Rates& r, const StagedPlan& p, DevStatus* st,
                        cudaStream_t s) {
  const RatesT<F2> r2 = rates_t<F2>(r);
  if (channel)
    k_fused_batch_x2<true><<<p.grid, p.threads, p.smem, s>>>(boxes, tasks, ntasks, ph, r2, p.S, st);
  else
    k_fused_batch_x2<false><<<p.grid, p.threads, p.smem, s>>>(boxes, tasks, ntasks, ph, r2, p.S, st);
  count_launch();
}

}  // namespace lbm
