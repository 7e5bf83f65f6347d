// lbm_internal.cuh - device-side types shared by the engine's CUDA sources.
//
// Data layout in HBM (one context = one box):
//   populations   f[q][z][y][x], q = 0..18, x fastest (structure of arrays),
//                 double (plain path) or float (shifted FP32 path), two
//                 buffers (current / next) of 19*N elements each;
//   node flags    isnodes[z][y][x] int32: particle id (0-based) for solid
//                 nodes, -1 for fluid, followed in the same allocation by
//                 the solid mask: one bit per node, rows (y, z) of sw 32-bit
//                 words (sw a multiple of 4, so a row is a 16-byte multiple);
//                 a second buffer keeps the flags of the previous step
//                 (isnodes0 of the reference);
//   forcing       for the low-wavenumber forcing, per-row coefficient tables
//                 rowtab[comp][kx][z][y] (complex) from which the body force
//                 at any node follows with five FMAs per component, plus a
//                 per-x twiddle table; two slots (previous, current step);
//   particles     (3, npart) FP64 vectors as in var_inc, plus per-particle
//                 link slabs link_code[p][cap] (node*32 + ipop),
//                 link_alpha[p][cap], link_f9[p][cap] and link_count[p].
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/lbm.h"

namespace lbm {

constexpr int NPOP = 19;

// D3Q19 lattice of the reference, B/para.f90:171-175
__host__ __device__ constexpr int cix(int q) {
  return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
       : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ciy(int q) {
  return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
       : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ciz(int q) {
  return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
       : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
// opposite direction (ipopp, B/para.f90:175)
__host__ __device__ constexpr int ipopp(int q) {
  return q == 0 ? 0
       : q <= 6 ? (q % 2 == 1 ? q + 1 : q - 1)
       : q <= 10 ? 17 - q
       : q <= 14 ? 25 - q
       : 33 - q;
}
static_assert(ipopp(7) == 10 && ipopp(8) == 9 && ipopp(11) == 14 && ipopp(12) == 13 &&
              ipopp(15) == 18 && ipopp(16) == 17 && ipopp(1) == 2 && ipopp(6) == 5,
              "opposite-direction table");

// MRT relaxation rates and constants (B/para.f90:96-169)
struct Rates {
  double s1, s2, s4, s9, s10, s13, s16;
  double omegepsl, omegepslj, omegxx;
};

// forcing evaluation mode inside the fluid kernels
enum ForceMode { FM_NONE = 0, FM_TABLE = 1, FM_CONST = 2 };

// Per-row forcing tables: for node (x, y, z) and component c,
//   F_c = Re B0 + 2 (Re B1 cos(2 pi x/nx) - Im B1 sin(..))
//             + 2 (Re B2 cos(4 pi x/nx) - Im B2 sin(..)),
// B_kx = rowtab[((c*3 + kx)*nz + z)*ny + y] (complex).
// The stochastic body force along one x-row (y, z) is a short Fourier series
// in x (kx = 0, 1, 2 are the only x wavenumbers of the forcing):
//   F_c(x) = k0 + k1 cos(2 pi x/nx) + k2 sin(2 pi x/nx) + k3 cos(4 pi x/nx) + k4 sin(4 pi x/nx)
// The table holds, per row, (k0..k4) of c = x, y, z at [5c .. 5c+4] and a
// zero in slot 15: 16 values, a multiple of 16 bytes in either precision.
constexpr int kRowCoef = 16;

template <typename T>
struct ForceView {
  int mode;                 // ForceMode
  const T* rowtab;          // [z*ny + y][kRowCoef] x-series coefficients, see below
  const T* xtw;             // per x: cos1, sin1, cos2, sin2
  T cfx, cfy, cfz;          // constant force (FM_CONST)
  // FP64 tables only: rowtab's coefficients as 64-bit fixed point at 2^-70
  // (|k| < 2^-7) and the twiddles at 2^-61, for the exact integer evaluation
  // of the series in the fixed-point fluid kernel
  const long long* rowtab_i = nullptr;
  const long long* xtw_i = nullptr;
};

struct Geometry {
  int nx, ny, nz;
  int nxh, nyh, nzh;
  long long N;
  int channel;
  int sw;                   // 32-bit words per row of the solid mask
  // FP64 populations stored as 64-bit fixed point (between fused steps of the
  // FP64 plain path; pop_from_fixed / pop_to_fixed) rather than as doubles
  int pop_fixed = 0;
};

// the solid mask that follows the N particle ids of a flag buffer
__host__ __device__ __forceinline__ const uint32_t* solid_mask(const int32_t* isnodes,
                                                               const Geometry& g) {
  return reinterpret_cast<const uint32_t*>(isnodes + g.N);
}
__host__ __device__ __forceinline__ const uint32_t* solid_mask_raw(const int32_t* isnodes,
                                                                   long long N) {
  return reinterpret_cast<const uint32_t*>(isnodes + N);
}
__device__ __forceinline__ bool is_solid(const uint32_t* mask, const Geometry& g, int row, int x) {
  return (mask[(size_t)row * g.sw + (x >> 5)] >> (x & 31)) & 1u;
}

// Particle state on the device, (3, npart_max) FP64 vectors, 0-based ids.
struct ParticleView {
  int npart;
  int cap;                  // link capacity per particle
  double rad, rhopart;
  const double* ypglb;
  const double* wp;
  const double* omgp;
};

// device error word values (first error wins)
struct DevStatus {
  int code;       // LBM_ERR_* or 0
  int where;      // kernel-specific detail (particle id, node ...)
};

__device__ inline void raise_error(DevStatus* st, int code, int where) {
  if (!st) return;
  if (atomicCAS(&st->code, 0, code) == 0) st->where = where;
}

}  // namespace lbm

// ---------------------------------------------------------------------------
// launch wrappers implemented in lbm_fluid.cu / lbm_particles.cu, called by
// the C ABI layer in lbm_capi.cu
namespace lbm {

// process-wide count of kernels this library has launched (lbm_kernel_launches)
void count_launch();

// fluid
template <typename T>
// fx: FP64 fixed-point moment sums; fcache/fcache_mode: the per-node force
// cache of the FP64 fixed-point kernel (k_fused in lbm_fluid.cu), mode 0 off
void launch_fused_step(const Geometry& g, const Rates& r, const T* fin, T* fout,
                       const int32_t* isnodes, const ForceView<T>& fprev,
                       const ForceView<T>& fnew, bool fx, T* fcache, int fcache_mode,
                       cudaStream_t s);
// the FP64 fixed-point step on populations stored in fixed point (fin and
// fout hold 64-bit integers at 2^-58; g.pop_fixed)
void launch_fused_fixed(const Geometry& g, const Rates& r, bool int_core, const double* fin,
                        double* fout,
                        const int32_t* isnodes, const ForceView<double>& fprev,
                        const ForceView<double>& fnew, double* fcache, int fcache_mode,
                        DevStatus* st, cudaStream_t s);
// n stored populations between FP64 and fixed point, in place; to fixed
// point, a value beyond |f| < 32 or not finite raises LBM_ERR_NONFINITE
void launch_pop_format(double* f, long long n, bool to_fixed, DevStatus* st, cudaStream_t s);
// twiddles at 2^-61 and the fixed-point row coefficients' range check
constexpr int kTwFix = 61;
// the same step with its rows staged through shared memory by bulk copies
// (lbm_staged.cu); periodic boxes with nx a multiple of 4
struct StagedPlan {
  int S = 0;            // input stages (rows in flight + 1)
  bool packed = false;  // FP32 pair kernel on f32x2 arithmetic
  int groups = 1;       // packed: consumer warp groups (rows in the collision at once)
  bool fx = false;      // FP64: exact fixed-point moment sums (collide_fx)
  int ctas_per_sm = 0;
  int grid = 0, threads = 0;
  size_t smem = 0;
};
template <typename T>
bool staged_eligible(const Geometry& g, int S, bool packed);
template <typename T>
int staged_max_stages(const Geometry& g);
template <typename T>
bool plan_fused_staged(const Geometry& g, int S, int ctas_per_sm, bool packed, int groups,
                       StagedPlan* plan, bool fx = false);
template <typename T>
void launch_fused_staged(const Geometry& g, const Rates& r, const T* fin, T* fout,
                         const int32_t* isnodes, const ForceView<T>& fprev,
                         const ForceView<T>& fnew, const StagedPlan& p, DevStatus* st,
                         cudaStream_t s);
// many boxes in one persistent FP32 kernel (lbm_batch.cu)
struct BatchBox {
  int nx, ny, nz, sw, N;
  float* f[2];                // population buffers
  const int32_t* flags[2];    // flag buffers (ids, then the solid mask)
  const float* rowtab[3];     // force coefficient slots
  const float* xtw;
  float cfx, cfy, cfz;        // constant force
};
struct BatchTask { int box, row0, nrows; };
// the step-dependent buffer and forcing choices, the same for every box of
// a batch advanced in lockstep
struct BatchPhase { int cur, fcur, prev_mode, prev_slot, new_mode, new_slot; };
int batch_task_rows(int nx, int ny);
bool batch_box_ok(const Geometry& g);
bool plan_batch(bool channel, int S, int groups, int ctas_per_sm, int ntasks, StagedPlan* plan);
void launch_fused_batch(bool channel, const BatchBox* boxes, const BatchTask* tasks, int ntasks,
                        const BatchPhase& ph, const Rates& r, const StagedPlan& p, DevStatus* st,
                        cudaStream_t s);

template <typename T>
void launch_macrovar(const Geometry& g, const T* f, const int32_t* isnodes,
                     const ForceView<T>& fv, const ParticleView& pv, T* rho, T* ux,
                     T* uy, T* uz, cudaStream_t s);
template <typename T>
void launch_collision(const Geometry& g, const Rates& r, T* f, const int32_t* isnodes,
                      const ForceView<T>& fv, const T* rho, const T* ux, const T* uy,
                      const T* uz, cudaStream_t s);
template <typename T>
void launch_streaming(const Geometry& g, const T* fin, T* fout, cudaStream_t s);
template <typename T>
void launch_rhoupdat_maxdiff(const Geometry& g, const T* f, T* rho, unsigned long long* maxbits,
                             cudaStream_t s);
template <typename T>
void launch_rhoupdat(const Geometry& g, const T* f, T* rho, cudaStream_t s);
template <typename T>
void launch_initpop(const Geometry& g, const double* ux, const double* uy,
                    const double* uz, T* f, T* rho, cudaStream_t s);
template <typename T>
void launch_aos_to_soa(const Geometry& g, const double* aos, T* soa, long long node0,
                       long long nnodes, cudaStream_t s);
template <typename T>
void launch_soa_to_aos(const Geometry& g, const T* soa, double* aos, long long node0,
                       long long nnodes, cudaStream_t s);
// SMs of the current device (queried once)
int sm_count();

// direct transfers between page-locked host memory (reference layout) and
// the SoA populations; `sms`: the device's SM count
template <typename T>
void launch_aos_host_to_soa(const double* aos_mapped, T* soa, long long N, int sms,
                            cudaStream_t s);
template <typename T>
void launch_soa_to_aos_host(const T* soa, double* aos_mapped, long long N, int sms,
                            cudaStream_t s);
// the same from the FP64 plain path's fixed-point storage (g.pop_fixed)
void launch_soa_fixed_to_aos_host(const long long* soa, double* aos_mapped, long long N, int sms,
                                  cudaStream_t s);
template <typename T>
void launch_convert(const double* in, T* out, long long n, cudaStream_t s);
template <typename T>
void launch_convert_back(const T* in, double* out, long long n, cudaStream_t s);
template <typename T>
void launch_force_field(const Geometry& g, const ForceView<T>& fv, double* fx, double* fy,
                        double* fz, cudaStream_t s);
template <typename T>
void launch_mass_momentum(const Geometry& g, const T* f, double* partial, int nblocks,
                          cudaStream_t s);

// forcing: advance the Ornstein-Uhlenbeck state by one FORCING call and build
// the per-row tables of the new force field
struct ForcingDev {
  int32_t iseedf, iyf, ivf[32];
  double b[450];   // b1r, b2r, b3r, each (6,5,5)
  double a[450];   // a1r, a2r, a3r
};
void launch_forcing_update(ForcingDev* st, double var, double tf, double pi2,
                           const double* kxr6, const double* kyr5, const double* kzr5,
                           cudaStream_t s);
template <typename T>
// ytw[jy][y], ztw[kz][z]: (cos, sin) of 2 pi k n / N for the five low
// wavenumbers of each axis, tabulated once per box (ytw in the populations'
// precision, ztw in FP64); ztab: the (kx, z) partial sums, T
// rowtab_i (FP64 only, may be null): the coefficients again as fixed point
// (ForceView::rowtab_i); a coefficient beyond its range raises LBM_ERR_STATE
// in status
void launch_forcing_tables(const Geometry& g, const ForcingDev* st, const T* ytw,
                           const double* ztw, T* rowtab, T* ztab, cudaStream_t s,
                           long long* rowtab_i = nullptr, DevStatus* status = nullptr);

// statistics (lbm_stats.cu): spectrum, dissipation and derivative moments
// of statistc; per-particle slip velocity
struct SpectrumWork;
void spectrum_free(SpectrumWork* w);
// rmsstat's fluid part (B/saveload.f90:1530-1730): out[0] fluid node count,
// out[1..3] mean u, out[4..6] rms u, out[7..9] mean vorticity, out[10..12]
// rms vorticity, all over fluid nodes (isnodes < 0)
template <typename T>
int fluid_rms_stats(const Geometry& g, const int32_t* isnodes, const T* ux, const T* uy,
                    const T* uz, SpectrumWork** pw, double* out, cudaStream_t s);
// per x-plane sums over (y, z) (nx x 12: u, v, w, uw, uv, vw, uu, vv, ww,
// rho, rho^2, count), all nodes or fluid nodes only
template <typename T>
int plane_sums(const Geometry& g, const int32_t* isnodes, int fluid_only, const T* rho,
               const T* ux, const T* uy, const T* uz, double* sums, cudaStream_t s);
// diag's max |u| over fluid nodes (B/saveload.f90:1357-1361)
template <typename T>
int fluid_vmax(const Geometry& g, const int32_t* isnodes, const T* ux, const T* uy, const T* uz,
               SpectrumWork** pw, double* vmax, cudaStream_t s);
template <typename T>
int spectrum_stats(const Geometry& g, double visc, const T* ux, const T* uy, const T* uz,
                   SpectrumWork** work, int nek_out, double* ek, double* dk, double* out,
                   cudaStream_t s);

// seeded divergence-free Gaussian velocity, E(k) ~ k^4 exp(-2 (k/k0)^2),
// per-component rms urms, into u[3][N] (device); synchronises s
int spectral_field(const Geometry& g, double k0, double urms, uint64_t seed, double* u,
                   cudaStream_t s);
int channel_loglaw_field(const Geometry& g, double visc, double* u, cudaStream_t s);
// per-block sums: mass, momentum x/y/z, population checksum, kinetic energy
template <typename T>
void launch_summary(const T* f, long long N, const T* ux, const T* uy, const T* uz,
                    double* partial, int nblocks, cudaStream_t s);

// particles
struct LinkSlab {
  int32_t* code;     // node*32 + ipop
  double* alpha;
  double* f9;
  int32_t* count;
  int cap;
  void* sweeps;      // per particle: nearest-image sweep events of the 3 axes (kSweepBytes)
  int32_t* sweep_ok; // per particle and axis: 1 if the sweep reached its fixed point
};
constexpr int kSweepBytes = 7 * 96;
// alpha_fp32: link fractions in single precision (the FP32 population path)
void launch_links(const Geometry& g, const ParticleView& pv, int32_t* isnodes,
                  LinkSlab ls, DevStatus* st, int alpha_fp32, cudaStream_t s,
                  bool sweeps_done = false);
template <typename T>
void launch_bounce_back(const Geometry& g, const ParticleView& pv, const T* f,
                        int pushed_layout, const int32_t* isnodes, LinkSlab ls,
                        double* fHIp, double* torqp, cudaStream_t s);
template <typename T>
void launch_bounce_scatter(const Geometry& g, const ParticleView& pv, T* f,
                           int pushed_layout, LinkSlab ls, cudaStream_t s,
                           DevStatus* st = nullptr);
template <typename T>
void launch_slip(const Geometry& g, const ParticleView& pv, const T* ux, const T* uy, const T* uz,
                 const int32_t* isnodes, double r_in, double r_out, double* slip, cudaStream_t s);
struct MoveState {
  double* ypglb; double* ypglbp; double* ypold;
  double* wp; double* wpp; double* omgp; double* omgpp;
  double* dwdt; double* domgdt; double* forcep; double* forcepp;
  double* torqp; double* torqpp; double* thetap; double* fHIp; double* flubp;
  int* first_move;  // device flag, cleared after the first beads_move
};
struct PartParams {
  double rad, mingap, mingap_w, fpc, stf0, stf1, stf0_w, stf1_w;
  double body_force_y, amp, aip, rho0, rhopart;
};
void launch_lubforce(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                     cudaStream_t s);
void launch_move(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                 cudaStream_t s);
void launch_redistribute(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                         DevStatus* st, cudaStream_t s);
// launch_move then launch_redistribute in two launches: the move and the wrap
// of a particle in one thread, then the overlap check (which also ends the
// first move).  The check only reports; with an aux stream it runs there,
// forked after the move by `fork` and recorded into `join`, beside the link
// kernels that follow on s (returns true: the caller joins `join`).
// With pv and ls, the same launch also runs beads_links' nearest-image
// sweeps of every moved particle (launch_links then skips them).
bool launch_move_redistribute(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                              DevStatus* st, cudaStream_t s, cudaStream_t aux = nullptr,
                              cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr,
                              const ParticleView* pv = nullptr, LinkSlab* ls = nullptr);
// refill events of one step: node index and particle id per event
struct FillList {
  int32_t* node;
  int32_t* part;
  int32_t* count;
  int cap;
};
// ---- particle step of many boxes per launch (lbm_batch) ---------------
// Everything one box's particle subroutines need for one buffer parity; the
// multi-box kernels take an array of these, blockIdx.y selecting the box.
struct BoxParticles {
  Geometry g;
  ParticleView pv;
  PartParams pp;
  MoveState ms;
  LinkSlab ls;
  FillList fl;
  float* f;               // populations after this step's stream + collide (pushed)
  int32_t* flags_cur;     // flags of this step
  int32_t* flags_next;    // flags the step builds
  DevStatus* st;
};
// one launch per kernel of the particle step (bounce-back through refill)
// for nb boxes of the array
void launch_particle_step_multi(const BoxParticles* boxes, int nb, int max_npart,
                                long long max_reset, cudaStream_t s);
// FORCING of many boxes into table slot `slot`, keeping each box's state
// before the update in `backup`
struct BoxForcing {
  Geometry g;
  ForcingDev* st;
  ForcingDev* backup;
  double var, tf, pi2;
  const double* kxr6; const double* kyr5; const double* kzr5;
  const float* ytw; const double* ztw;
  float* ztab;
  float* rowtab[3];
};
void launch_forcing_multi(const BoxForcing* boxes, int nb, int max_nz, long long max_rows,
                          int slot, cudaStream_t s);

template <typename T>
void launch_filling(const Geometry& g, const ParticleView& pv, const PartParams& pp,
                    const double* ypglbp, const double* wpp, const double* omgpp,
                    const int32_t* isnodes, const int32_t* isnodes0, T* f, FillList fl,
                    DevStatus* st, cudaStream_t s);

// initpartvel: wp (3, npart) at the centres y (3, npart) from the velocity
// fields; *bad (set to npart by the caller) becomes the smallest index of a
// centre outside the interpolation range
template <typename T>
void launch_initpartvel(const Geometry& g, const T* ux, const T* uy, const T* uz,
                        const double* y, int npart, double* wp, int* bad, cudaStream_t s);

}  // namespace lbm
